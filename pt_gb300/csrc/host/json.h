// json.h — a small JSON reader for glTF 2.0 documents.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace pth {

struct Json {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    bool has(const std::string& k) const { return kind == OBJ && obj.count(k) > 0; }
    const Json& operator[](const std::string& k) const
    {
        static const Json null_value;
        if (kind != OBJ)
            return null_value;
        auto it = obj.find(k);
        return it == obj.end() ? null_value : it->second;
    }
    const Json& operator[](size_t i) const
    {
        static const Json null_value;
        if (kind != ARR || i >= arr.size())
            return null_value;
        return arr[i];
    }
    size_t size() const { return kind == ARR ? arr.size() : (kind == OBJ ? obj.size() : 0); }
    double number(double def) const { return kind == NUM ? num : def; }
    int64_t integer(int64_t def) const { return kind == NUM ? (int64_t)num : def; }
};

class JsonParser {
  public:
    explicit JsonParser(const std::string& text) : s(text) {}
    Json parse()
    {
        Json v = value();
        ws();
        if (i != s.size())
            fail("trailing characters");
        return v;
    }

  private:
    const std::string& s;
    size_t i = 0;
    int depth = 0;

    [[noreturn]] void fail(const char* what) { throw std::runtime_error(std::string("JSON: ") + what + " at offset " + std::to_string(i)); }
    void ws()
    {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r'))
            i++;
    }
    bool lit(const char* w)
    {
        size_t n = std::char_traits<char>::length(w);
        if (s.compare(i, n, w) == 0) {
            i += n;
            return true;
        }
        return false;
    }
    Json value()
    {
        if (++depth > 256)
            fail("nesting too deep");
        ws();
        if (i >= s.size())
            fail("unexpected end");
        Json v;
        char c = s[i];
        if (c == '{') {
            v.kind = Json::OBJ;
            i++;
            ws();
            if (i < s.size() && s[i] == '}') {
                i++;
            } else {
                while (true) {
                    ws();
                    if (i >= s.size() || s[i] != '"')
                        fail("expected key");
                    std::string k = string();
                    ws();
                    if (i >= s.size() || s[i] != ':')
                        fail("expected ':'");
                    i++;
                    v.obj[k] = value();
                    ws();
                    if (i < s.size() && s[i] == ',') {
                        i++;
                        continue;
                    }
                    if (i < s.size() && s[i] == '}') {
                        i++;
                        break;
                    }
                    fail("expected ',' or '}'");
                }
            }
        } else if (c == '[') {
            v.kind = Json::ARR;
            i++;
            ws();
            if (i < s.size() && s[i] == ']') {
                i++;
            } else {
                while (true) {
                    v.arr.push_back(value());
                    ws();
                    if (i < s.size() && s[i] == ',') {
                        i++;
                        continue;
                    }
                    if (i < s.size() && s[i] == ']') {
                        i++;
                        break;
                    }
                    fail("expected ',' or ']'");
                }
            }
        } else if (c == '"') {
            v.kind = Json::STR;
            v.str = string();
        } else if (lit("true")) {
            v.kind = Json::BOOL;
            v.b = true;
        } else if (lit("false")) {
            v.kind = Json::BOOL;
        } else if (lit("null")) {
            v.kind = Json::NUL;
        } else {
            size_t start = i;
            while (i < s.size() && (std::isdigit((unsigned char)s[i]) || s[i] == '-' || s[i] == '+' || s[i] == '.' || s[i] == 'e' || s[i] == 'E'))
                i++;
            if (start == i)
                fail("unexpected character");
            v.kind = Json::NUM;
            try {
                v.num = std::stod(s.substr(start, i - start));
            } catch (...) {
                fail("bad number");
            }
        }
        depth--;
        return v;
    }
    std::string string()
    {
        i++; // opening quote
        std::string out;
        while (i < s.size() && s[i] != '"') {
            char c = s[i++];
            if (c == '\\') {
                if (i >= s.size())
                    fail("bad escape");
                char e = s[i++];
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
                    if (i + 4 > s.size())
                        fail("bad \\u escape");
                    unsigned cp = (unsigned)std::stoul(s.substr(i, 4), nullptr, 16);
                    i += 4;
                    if (cp < 0x80) {
                        out += (char)cp;
                    } else if (cp < 0x800) {
                        out += (char)(0xC0 | (cp >> 6));
                        out += (char)(0x80 | (cp & 0x3F));
                    } else {
                        out += (char)(0xE0 | (cp >> 12));
                        out += (char)(0x80 | ((cp >> 6) & 0x3F));
                        out += (char)(0x80 | (cp & 0x3F));
                    }
                    break;
                }
                default: fail("bad escape");
                }
            } else {
                out += c;
            }
        }
        if (i >= s.size())
            fail("unterminated string");
        i++;
        return out;
    }
};

} // namespace pth
