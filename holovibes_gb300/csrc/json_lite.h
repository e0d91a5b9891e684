// A small JSON reader / writer (objects keep insertion order) shared by the compute-settings
// loader and the .holo footer. Numbers are doubles; \u escapes are decoded to UTF-8.
#pragma once

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace hv {
namespace json {

struct Value
{
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Value> arr;
    std::vector<std::pair<std::string, Value>> obj;  // insertion order

    const Value* find(const std::string& k) const
    {
        for (const auto& kv : obj)
            if (kv.first == k)
                return &kv.second;
        return nullptr;
    }
    Value* find(const std::string& k)
    {
        for (auto& kv : obj)
            if (kv.first == k)
                return &kv.second;
        return nullptr;
    }
};

struct Parser
{
    const char* p;
    const char* end;
    std::string err;

    void ws()
    {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r'))
            ++p;
    }
    bool fail(const char* m)
    {
        if (err.empty())
            err = m;
        return false;
    }
    bool lit(const char* s)
    {
        const size_t n = std::strlen(s);
        if (static_cast<size_t>(end - p) < n || std::strncmp(p, s, n) != 0)
            return false;
        p += n;
        return true;
    }
    bool string(std::string& out)
    {
        if (p >= end || *p != '"')
            return fail("expected string");
        ++p;
        while (p < end && *p != '"')
        {
            char c = *p++;
            if (c == '\\')
            {
                if (p >= end)
                    return fail("bad escape");
                const char e = *p++;
                switch (e)
                {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u':
                {
                    if (end - p < 4)
                        return fail("bad unicode escape");
                    unsigned int cp = 0;
                    for (int i = 0; i < 4; ++i)
                    {
                        const char h = p[i];
                        cp <<= 4;
                        if (h >= '0' && h <= '9')
                            cp |= static_cast<unsigned int>(h - '0');
                        else if (h >= 'a' && h <= 'f')
                            cp |= static_cast<unsigned int>(h - 'a' + 10);
                        else if (h >= 'A' && h <= 'F')
                            cp |= static_cast<unsigned int>(h - 'A' + 10);
                        else
                            return fail("bad unicode escape");
                    }
                    p += 4;
                    if (cp < 0x80)
                        out += static_cast<char>(cp);
                    else if (cp < 0x800)
                    {
                        out += static_cast<char>(0xC0 | (cp >> 6));
                        out += static_cast<char>(0x80 | (cp & 0x3F));
                    }
                    else
                    {
                        out += static_cast<char>(0xE0 | (cp >> 12));
                        out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
                        out += static_cast<char>(0x80 | (cp & 0x3F));
                    }
                    break;
                }
                default: return fail("bad escape");
                }
            }
            else
                out += c;
        }
        if (p >= end)
            return fail("unterminated string");
        ++p;
        return true;
    }
    bool value(Value& v, int depth)
    {
        if (depth > 64)
            return fail("nesting too deep");
        ws();
        if (p >= end)
            return fail("unexpected end");
        const char c = *p;
        if (c == '{')
        {
            ++p;
            v.kind = Value::Object;
            ws();
            if (p < end && *p == '}')
            {
                ++p;
                return true;
            }
            for (;;)
            {
                ws();
                std::string k;
                if (!string(k))
                    return false;
                ws();
                if (p >= end || *p != ':')
                    return fail("expected ':'");
                ++p;
                Value child;
                if (!value(child, depth + 1))
                    return false;
                Value* existing = v.find(k);
                if (existing)
                    *existing = std::move(child);
                else
                    v.obj.emplace_back(std::move(k), std::move(child));
                ws();
                if (p < end && *p == ',')
                {
                    ++p;
                    continue;
                }
                if (p < end && *p == '}')
                {
                    ++p;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[')
        {
            ++p;
            v.kind = Value::Array;
            ws();
            if (p < end && *p == ']')
            {
                ++p;
                return true;
            }
            for (;;)
            {
                Value child;
                if (!value(child, depth + 1))
                    return false;
                v.arr.push_back(std::move(child));
                ws();
                if (p < end && *p == ',')
                {
                    ++p;
                    continue;
                }
                if (p < end && *p == ']')
                {
                    ++p;
                    return true;
                }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"')
        {
            v.kind = Value::String;
            return string(v.str);
        }
        if (lit("true"))
        {
            v.kind = Value::Bool;
            v.b = true;
            return true;
        }
        if (lit("false"))
        {
            v.kind = Value::Bool;
            v.b = false;
            return true;
        }
        if (lit("null"))
        {
            v.kind = Value::Null;
            return true;
        }
        // number
        const char* s = p;
        if (p < end && (*p == '-' || *p == '+'))
            ++p;
        while (p < end && (std::isdigit(static_cast<unsigned char>(*p)) || *p == '.' || *p == 'e' || *p == 'E' ||
                           *p == '-' || *p == '+'))
            ++p;
        if (p == s)
            return fail("unexpected character");
        std::string num(s, p);
        char* e = nullptr;
        v.kind = Value::Number;
        v.num = std::strtod(num.c_str(), &e);
        if (!e || *e != '\0')
            return fail("bad number");
        return true;
    }
};

inline bool parse(const char* text, Value& out, std::string& err)
{
    Parser ps{text, text + std::strlen(text), {}};
    if (!ps.value(out, 0))
    {
        err = ps.err;
        return false;
    }
    ps.ws();
    if (ps.p != ps.end)
    {
        err = "trailing characters";
        return false;
    }
    return true;
}


// Compact serialisation (no whitespace), numbers with 17 significant digits (integers exactly).
inline void dump(const Value& v, std::string& out)
{
    switch (v.kind)
    {
    case Value::Null: out += "null"; break;
    case Value::Bool: out += v.b ? "true" : "false"; break;
    case Value::Number:
    {
        char buf[40];
        if (std::fabs(v.num) < 9.0e15 && v.num == static_cast<double>(static_cast<long long>(v.num)))
            std::snprintf(buf, sizeof(buf), "%lld", static_cast<long long>(v.num));
        else
            std::snprintf(buf, sizeof(buf), "%.17g", v.num);
        out += buf;
        break;
    }
    case Value::String:
        out += '"';
        for (const char c : v.str)
        {
            switch (c)
            {
            case '"': out += "\\\""; break;
            case '\\': out += "\\\\"; break;
            case '\n': out += "\\n"; break;
            case '\r': out += "\\r"; break;
            case '\t': out += "\\t"; break;
            default:
                if (static_cast<unsigned char>(c) < 0x20)
                {
                    char buf[8];
                    std::snprintf(buf, sizeof(buf), "\\u%04x", static_cast<unsigned int>(static_cast<unsigned char>(c)));
                    out += buf;
                }
                else
                    out += c;
            }
        }
        out += '"';
        break;
    case Value::Array:
        out += '[';
        for (size_t i = 0; i < v.arr.size(); ++i)
        {
            if (i)
                out += ',';
            dump(v.arr[i], out);
        }
        out += ']';
        break;
    case Value::Object:
        out += '{';
        for (size_t i = 0; i < v.obj.size(); ++i)
        {
            if (i)
                out += ',';
            Value k;
            k.kind = Value::String;
            k.str = v.obj[i].first;
            dump(k, out);
            out += ':';
            dump(v.obj[i].second, out);
        }
        out += '}';
        break;
    }
}

}  // namespace json
}  // namespace hv
