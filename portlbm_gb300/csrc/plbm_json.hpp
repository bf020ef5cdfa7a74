// plbm_json.hpp — the small JSON subset settings.json needs (objects, arrays, strings,
// numbers, booleans, null), for reading and writing settings like
// file_interaction::json_to_properties / properties_to_json (file_interaction.cpp:11-69).
#pragma once

#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace plbm {

struct JsonError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

struct Json {
    enum Type { NUL, BOOL, NUMBER, STRING, ARRAY, OBJECT } type = NUL;
    bool b = false;
    double num = 0;
    bool is_integer = false;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    const Json *find(const std::string &k) const
    {
        for (const auto &kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
    // nlohmann::json::at semantics: a missing key is an error naming the key.
    const Json &at(const std::string &k) const
    {
        if (type != OBJECT) throw JsonError("type_error: cannot use at() with " + type_name());
        const Json *v = find(k);
        if (!v) throw JsonError("out_of_range: key '" + k + "' not found");
        return *v;
    }
    std::string type_name() const
    {
        static const char *n[] = { "null", "boolean", "number", "string", "array", "object" };
        return n[type];
    }
    unsigned as_unsigned() const
    {
        if (type != NUMBER) throw JsonError("type_error: type must be number, but is " + type_name());
        return (unsigned)(long long)num;
    }
    double as_double() const
    {
        if (type != NUMBER) throw JsonError("type_error: type must be number, but is " + type_name());
        return num;
    }
    bool as_bool() const
    {
        if (type != BOOL) throw JsonError("type_error: type must be boolean, but is " + type_name());
        return b;
    }
    const std::string &as_string() const
    {
        if (type != STRING) throw JsonError("type_error: type must be string, but is " + type_name());
        return str;
    }
    Json &set(const std::string &k)
    {
        type = OBJECT;
        for (auto &kv : obj)
            if (kv.first == k) return kv.second;
        obj.emplace_back(k, Json());
        return obj.back().second;
    }
};

class JsonParser {
  public:
    explicit JsonParser(const std::string &s) : s_(s) {}
    Json parse()
    {
        Json v = value();
        ws();
        if (i_ != s_.size()) fail("unexpected trailing characters");
        return v;
    }

  private:
    const std::string &s_;
    size_t i_ = 0;

    [[noreturn]] void fail(const char *what)
    {
        throw JsonError(std::string("parse_error at byte ") + std::to_string(i_) + ": " + what);
    }
    void ws()
    {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\n' || s_[i_] == '\r' || s_[i_] == '\t')) ++i_;
    }
    Json value()
    {
        ws();
        if (i_ >= s_.size()) fail("unexpected end of input");
        const char c = s_[i_];
        if (c == '{') return object();
        if (c == '[') return array();
        if (c == '"') { Json j; j.type = Json::STRING; j.str = string(); return j; }
        if (c == 't' || c == 'f' || c == 'n') return literal();
        return number();
    }
    Json object()
    {
        Json j; j.type = Json::OBJECT; ++i_;
        ws();
        if (i_ < s_.size() && s_[i_] == '}') { ++i_; return j; }
        for (;;) {
            ws();
            if (i_ >= s_.size() || s_[i_] != '"') fail("expected string key");
            std::string k = string();
            ws();
            if (i_ >= s_.size() || s_[i_] != ':') fail("expected ':'");
            ++i_;
            j.obj.emplace_back(std::move(k), value());
            ws();
            if (i_ < s_.size() && s_[i_] == ',') { ++i_; continue; }
            if (i_ < s_.size() && s_[i_] == '}') { ++i_; return j; }
            fail("expected ',' or '}'");
        }
    }
    Json array()
    {
        Json j; j.type = Json::ARRAY; ++i_;
        ws();
        if (i_ < s_.size() && s_[i_] == ']') { ++i_; return j; }
        for (;;) {
            j.arr.push_back(value());
            ws();
            if (i_ < s_.size() && s_[i_] == ',') { ++i_; continue; }
            if (i_ < s_.size() && s_[i_] == ']') { ++i_; return j; }
            fail("expected ',' or ']'");
        }
    }
    std::string string()
    {
        ++i_;
        std::string out;
        while (i_ < s_.size() && s_[i_] != '"') {
            char c = s_[i_++];
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
                default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (i_ >= s_.size()) fail("unterminated string");
        ++i_;
        return out;
    }
    Json literal()
    {
        Json j;
        if (s_.compare(i_, 4, "true") == 0) { j.type = Json::BOOL; j.b = true; i_ += 4; }
        else if (s_.compare(i_, 5, "false") == 0) { j.type = Json::BOOL; j.b = false; i_ += 5; }
        else if (s_.compare(i_, 4, "null") == 0) { i_ += 4; }
        else fail("invalid literal");
        return j;
    }
    Json number()
    {
        const char *b = s_.c_str() + i_;
        char *e = nullptr;
        double v = std::strtod(b, &e);
        if (e == b) fail("invalid value");
        Json j; j.type = Json::NUMBER; j.num = v;
        j.is_integer = std::string(b, (size_t)(e - b)).find_first_of(".eE") == std::string::npos;
        i_ += (size_t)(e - b);
        return j;
    }
};

inline void json_escape(std::string &out, const std::string &s)
{
    out += '"';
    for (char c : s) {
        if (c == '"' || c == '\\') { out += '\\'; out += c; }
        else if (c == '\n') out += "\\n";
        else out += c;
    }
    out += '"';
}

// Serialises with 4-space indentation like `file << std::setw(4) << json` (keys in insertion order).
inline void json_dump(std::string &out, const Json &j, int indent = 0)
{
    char buf[64];
    switch (j.type) {
    case Json::NUL: out += "null"; break;
    case Json::BOOL: out += j.b ? "true" : "false"; break;
    case Json::NUMBER:
        if (j.is_integer) {
            std::snprintf(buf, sizeof buf, "%lld", (long long)j.num);
        } else {
            // shortest representation that reads back to the same double, as nlohmann writes
            for (int prec = 15; prec <= 17; ++prec) {
                std::snprintf(buf, sizeof buf, "%.*g", prec, j.num);
                if (std::strtod(buf, nullptr) == j.num) break;
            }
            if (!std::strpbrk(buf, ".eEn")) std::strcat(buf, ".0");
        }
        out += buf;
        break;
    case Json::STRING: json_escape(out, j.str); break;
    case Json::ARRAY:
        out += "[\n";
        for (size_t k = 0; k < j.arr.size(); ++k) {
            out.append((size_t)(indent + 4), ' ');
            json_dump(out, j.arr[k], indent + 4);
            out += k + 1 < j.arr.size() ? ",\n" : "\n";
        }
        out.append((size_t)indent, ' ');
        out += "]";
        break;
    case Json::OBJECT:
        out += "{\n";
        for (size_t k = 0; k < j.obj.size(); ++k) {
            out.append((size_t)(indent + 4), ' ');
            json_escape(out, j.obj[k].first);
            out += ": ";
            json_dump(out, j.obj[k].second, indent + 4);
            out += k + 1 < j.obj.size() ? ",\n" : "\n";
        }
        out.append((size_t)indent, ' ');
        out += "}";
        break;
    }
}

inline Json jnum(double v, bool integer) { Json j; j.type = Json::NUMBER; j.num = v; j.is_integer = integer; return j; }
inline Json jstr(const std::string &s) { Json j; j.type = Json::STRING; j.str = s; return j; }
inline Json jbool(bool b) { Json j; j.type = Json::BOOL; j.b = b; return j; }

}  // namespace plbm
