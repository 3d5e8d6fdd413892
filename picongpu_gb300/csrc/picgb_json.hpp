// A small JSON value with a writer and a parser, for the openPMD series index of
// the checkpoint files (picgb_openpmd.cu).  Objects keep their insertion order;
// numbers are doubles (exact for the integers an index holds, < 2^53).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace picgb::json
{
    class Value
    {
    public:
        enum Kind
        {
            Null,
            Bool,
            Number,
            String,
            Array,
            Object
        };

        Value() = default;
        Value(bool b) : kind_(Bool), b_(b) {}
        Value(double d) : kind_(Number), d_(d) {}
        Value(int i) : kind_(Number), d_(i) {}
        Value(unsigned i) : kind_(Number), d_(i) {}
        Value(int64_t i) : kind_(Number), d_(double(i)) {}
        Value(uint64_t i) : kind_(Number), d_(double(i)) {}
        Value(char const* s) : kind_(String), s_(s) {}
        Value(std::string s) : kind_(String), s_(std::move(s)) {}

        static Value array() { return Value(Array); }
        static Value object() { return Value(Object); }

        Kind kind() const { return kind_; }
        bool isObject() const { return kind_ == Object; }
        bool isArray() const { return kind_ == Array; }
        bool isNumber() const { return kind_ == Number; }
        bool isString() const { return kind_ == String; }

        double number() const
        {
            need(Number, "a number");
            return d_;
        }
        std::string const& string() const
        {
            need(String, "a string");
            return s_;
        }
        std::vector<Value> const& items() const
        {
            need(Array, "an array");
            return a_;
        }
        std::vector<std::pair<std::string, Value>> const& members() const
        {
            need(Object, "an object");
            return o_;
        }

        // Object member, created if absent.  The reference stays valid until the next
        // member is added to this same object.
        Value& operator[](std::string const& key)
        {
            need(Object, "an object");
            for(auto& kv : o_)
                if(kv.first == key)
                    return kv.second;
            o_.emplace_back(key, Value());
            return o_.back().second;
        }
        // object member or nullptr
        Value const* find(std::string const& key) const
        {
            if(kind_ != Object)
                return nullptr;
            for(auto const& kv : o_)
                if(kv.first == key)
                    return &kv.second;
            return nullptr;
        }
        // object member; throws when absent
        Value const& at(std::string const& key) const
        {
            Value const* v = find(key);
            if(!v)
                throw std::runtime_error("missing key '" + key + "'");
            return *v;
        }
        Value& push(Value v)
        {
            need(Array, "an array");
            a_.push_back(std::move(v));
            return a_.back();
        }

        void write(std::string& out, int indent = 0) const
        {
            switch(kind_)
            {
            case Null:
                out += "null";
                break;
            case Bool:
                out += b_ ? "true" : "false";
                break;
            case Number:
                writeNumber(out, d_);
                break;
            case String:
                writeString(out, s_);
                break;
            case Array:
                out += '[';
                for(size_t i = 0; i < a_.size(); ++i)
                {
                    if(i)
                        out += ", ";
                    a_[i].write(out, indent);
                }
                out += ']';
                break;
            case Object:
                out += "{";
                for(size_t i = 0; i < o_.size(); ++i)
                {
                    out += i ? ",\n" : "\n";
                    out.append(size_t(indent + 2), ' ');
                    writeString(out, o_[i].first);
                    out += ": ";
                    o_[i].second.write(out, indent + 2);
                }
                if(!o_.empty())
                {
                    out += '\n';
                    out.append(size_t(indent), ' ');
                }
                out += '}';
                break;
            }
        }

        static Value parse(std::string const& text)
        {
            size_t i = 0;
            Value v = parseValue(text, i);
            skipWs(text, i);
            if(i != text.size())
                throw std::runtime_error("trailing characters after the JSON value");
            return v;
        }

    private:
        explicit Value(Kind k) : kind_(k) {}

        void need(Kind k, char const* what) const
        {
            if(kind_ != k)
                throw std::runtime_error(std::string("JSON value is not ") + what);
        }

        static void writeNumber(std::string& out, double d)
        {
            char buf[40];
            if(!std::isfinite(d))
                throw std::runtime_error("JSON cannot hold a non-finite number");
            if(d == std::floor(d) && std::fabs(d) < 9007199254740992.0)
                std::snprintf(buf, sizeof(buf), "%lld", (long long) d);
            else
                std::snprintf(buf, sizeof(buf), "%.17g", d);
            out += buf;
        }

        static void writeString(std::string& out, std::string const& s)
        {
            out += '"';
            for(unsigned char c : s)
            {
                if(c == '"' || c == '\\')
                {
                    out += '\\';
                    out += char(c);
                }
                else if(c < 0x20)
                {
                    char buf[8];
                    std::snprintf(buf, sizeof(buf), "\\u%04x", c);
                    out += buf;
                }
                else
                    out += char(c);
            }
            out += '"';
        }

        static void skipWs(std::string const& t, size_t& i)
        {
            while(i < t.size() && (t[i] == ' ' || t[i] == '\n' || t[i] == '\r' || t[i] == '\t'))
                ++i;
        }

        static void expect(std::string const& t, size_t& i, char const* word)
        {
            for(char const* w = word; *w; ++w, ++i)
                if(i >= t.size() || t[i] != *w)
                    throw std::runtime_error(std::string("malformed JSON: expected '") + word + "'");
        }

        static std::string parseString(std::string const& t, size_t& i)
        {
            if(i >= t.size() || t[i] != '"')
                throw std::runtime_error("malformed JSON: expected a string");
            ++i;
            std::string s;
            while(true)
            {
                if(i >= t.size())
                    throw std::runtime_error("malformed JSON: unterminated string");
                char c = t[i++];
                if(c == '"')
                    return s;
                if(c != '\\')
                {
                    s += c;
                    continue;
                }
                if(i >= t.size())
                    throw std::runtime_error("malformed JSON: bad escape");
                char e = t[i++];
                switch(e)
                {
                case '"':
                case '\\':
                case '/':
                    s += e;
                    break;
                case 'n':
                    s += '\n';
                    break;
                case 't':
                    s += '\t';
                    break;
                case 'r':
                    s += '\r';
                    break;
                case 'b':
                    s += '\b';
                    break;
                case 'f':
                    s += '\f';
                    break;
                case 'u':
                {
                    if(i + 4 > t.size())
                        throw std::runtime_error("malformed JSON: bad \\u escape");
                    unsigned cp = unsigned(std::strtoul(t.substr(i, 4).c_str(), nullptr, 16));
                    i += 4;
                    if(cp < 0x80)
                        s += char(cp);
                    else if(cp < 0x800)
                    {
                        s += char(0xC0 | (cp >> 6));
                        s += char(0x80 | (cp & 0x3F));
                    }
                    else
                    {
                        s += char(0xE0 | (cp >> 12));
                        s += char(0x80 | ((cp >> 6) & 0x3F));
                        s += char(0x80 | (cp & 0x3F));
                    }
                    break;
                }
                default:
                    throw std::runtime_error("malformed JSON: bad escape");
                }
            }
        }

        static Value parseValue(std::string const& t, size_t& i)
        {
            skipWs(t, i);
            if(i >= t.size())
                throw std::runtime_error("malformed JSON: unexpected end");
            char c = t[i];
            if(c == '{')
            {
                ++i;
                Value v = object();
                skipWs(t, i);
                if(i < t.size() && t[i] == '}')
                {
                    ++i;
                    return v;
                }
                while(true)
                {
                    skipWs(t, i);
                    std::string key = parseString(t, i);
                    skipWs(t, i);
                    expect(t, i, ":");
                    v.o_.emplace_back(std::move(key), parseValue(t, i));
                    skipWs(t, i);
                    if(i < t.size() && t[i] == ',')
                    {
                        ++i;
                        continue;
                    }
                    expect(t, i, "}");
                    return v;
                }
            }
            if(c == '[')
            {
                ++i;
                Value v = array();
                skipWs(t, i);
                if(i < t.size() && t[i] == ']')
                {
                    ++i;
                    return v;
                }
                while(true)
                {
                    v.a_.push_back(parseValue(t, i));
                    skipWs(t, i);
                    if(i < t.size() && t[i] == ',')
                    {
                        ++i;
                        continue;
                    }
                    expect(t, i, "]");
                    return v;
                }
            }
            if(c == '"')
                return Value(parseString(t, i));
            if(c == 't')
            {
                expect(t, i, "true");
                return Value(true);
            }
            if(c == 'f')
            {
                expect(t, i, "false");
                return Value(false);
            }
            if(c == 'n')
            {
                expect(t, i, "null");
                return Value();
            }
            char const* start = t.c_str() + i;
            char* end = nullptr;
            double d = std::strtod(start, &end);
            if(end == start)
                throw std::runtime_error("malformed JSON: unexpected character");
            i += size_t(end - start);
            return Value(d);
        }

        Kind kind_ = Null;
        bool b_ = false;
        double d_ = 0.0;
        std::string s_;
        std::vector<Value> a_;
        std::vector<std::pair<std::string, Value>> o_;
    };
} // namespace picgb::json
