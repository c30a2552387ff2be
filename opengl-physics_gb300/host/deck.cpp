// deck.cpp -- a TOML-subset parser and the dotted-path accessors of fw::Deck.
#include "deck.hpp"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <sstream>
#include <stdexcept>

namespace fw {

namespace {

using Ptr = std::shared_ptr<TomlValue>;

Ptr make(TomlValue::Kind k) {
    auto v = std::make_shared<TomlValue>();
    v->kind = k;
    return v;
}

class Parser {
public:
    Parser(std::string_view text, std::string name) : s_(text), name_(std::move(name)) {}

    Ptr Parse() {
        Ptr root = make(TomlValue::Table);
        TomlValue* cur = root.get();
        for (;;) {
            SkipWsNl();
            if (Eof()) break;
            if (Peek() == '[') {
                const bool aot = pos_ + 1 < s_.size() && s_[pos_ + 1] == '[';
                pos_ += aot ? 2 : 1;
                SkipWs();
                std::vector<std::string> key = ParseKey();
                SkipWs();
                Expect(']');
                if (aot) Expect(']');
                cur = aot ? OpenArrayTable(root.get(), key) : OpenTable(root.get(), key);
                EndOfLine();
                continue;
            }
            std::vector<std::string> key = ParseKey();
            SkipWs();
            Expect('=');
            SkipWs();
            Ptr val = ParseValue();
            Assign(cur, key, val);
            EndOfLine();
        }
        return root;
    }

private:
    [[noreturn]] void Fail(const std::string& what) {
        std::ostringstream ss;
        ss << "Deck: parse error in " << name_ << ": " << what << " at line " << line_;
        throw std::runtime_error(ss.str());
    }
    bool Eof() const { return pos_ >= s_.size(); }
    char Peek() const { return Eof() ? '\0' : s_[pos_]; }
    char Get() {
        const char c = Peek();
        ++pos_;
        if (c == '\n') ++line_;
        return c;
    }
    void Expect(char c) {
        if (Peek() != c) Fail(std::string("expected '") + c + "'");
        Get();
    }
    void SkipWs() {
        while (!Eof() && (Peek() == ' ' || Peek() == '\t')) ++pos_;
    }
    void SkipComment() {
        if (Peek() == '#')
            while (!Eof() && Peek() != '\n') ++pos_;
    }
    void SkipWsNl() {
        for (;;) {
            SkipWs();
            SkipComment();
            if (Peek() == '\n' || Peek() == '\r') {
                Get();
                continue;
            }
            break;
        }
    }
    void EndOfLine() {
        SkipWs();
        SkipComment();
        if (Eof()) return;
        if (Peek() == '\r') Get();
        if (Peek() != '\n') Fail("unexpected text after value");
        Get();
    }

    std::vector<std::string> ParseKey() {
        std::vector<std::string> parts;
        for (;;) {
            SkipWs();
            if (Peek() == '"' || Peek() == '\'') {
                parts.push_back(ParseStringRaw());
            } else {
                std::string k;
                while (!Eof() && (std::isalnum((unsigned char)Peek()) || Peek() == '_' || Peek() == '-')) k += Get();
                if (k.empty()) Fail("expected a key");
                parts.push_back(k);
            }
            SkipWs();
            if (Peek() != '.') break;
            Get();
        }
        return parts;
    }

    static TomlValue* Child(TomlValue* t, const std::string& k, bool create) {
        auto it = t->table.find(k);
        if (it != t->table.end()) return it->second.get();
        if (!create) return nullptr;
        Ptr v = make(TomlValue::Table);
        t->table[k] = v;
        return v.get();
    }

    TomlValue* Descend(TomlValue* t, const std::vector<std::string>& key, size_t upto) {
        for (size_t i = 0; i < upto; ++i) {
            TomlValue* c = Child(t, key[i], true);
            if (c->kind == TomlValue::Array) {
                if (c->array.empty() || c->array.back()->kind != TomlValue::Table) Fail("key is not a table");
                c = c->array.back().get();
            } else if (c->kind != TomlValue::Table) {
                Fail("key '" + key[i] + "' is not a table");
            }
            t = c;
        }
        return t;
    }

    TomlValue* OpenTable(TomlValue* root, const std::vector<std::string>& key) {
        return Descend(root, key, key.size());
    }

    TomlValue* OpenArrayTable(TomlValue* root, const std::vector<std::string>& key) {
        TomlValue* parent = Descend(root, key, key.size() - 1);
        auto it = parent->table.find(key.back());
        Ptr arr;
        if (it == parent->table.end()) {
            arr = make(TomlValue::Array);
            parent->table[key.back()] = arr;
        } else {
            arr = it->second;
            if (arr->kind != TomlValue::Array) Fail("key '" + key.back() + "' is not an array of tables");
        }
        Ptr t = make(TomlValue::Table);
        arr->array.push_back(t);
        return t.get();
    }

    void Assign(TomlValue* cur, const std::vector<std::string>& key, const Ptr& val) {
        TomlValue* t = Descend(cur, key, key.size() - 1);
        if (t->table.count(key.back())) Fail("duplicate key '" + key.back() + "'");
        t->table[key.back()] = val;
    }

    std::string ParseStringRaw() {
        const char q = Get();
        const bool multi = Peek() == q && pos_ + 1 < s_.size() && s_[pos_ + 1] == q;
        if (multi) {
            pos_ += 2;
            if (Peek() == '\r') Get();
            if (Peek() == '\n') Get();
        }
        std::string out;
        for (;;) {
            if (Eof()) Fail("unterminated string");
            const char c = Get();
            if (c == q) {
                if (!multi) return out;
                if (Peek() == q && pos_ + 1 < s_.size() && s_[pos_ + 1] == q) {
                    pos_ += 2;
                    return out;
                }
                out += c;
                continue;
            }
            if (c == '\n' && !multi) Fail("newline in string");
            if (c == '\\' && q == '"') {
                const char e = Get();
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case '"': out += '"'; break;
                    case '\\': out += '\\'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    default: Fail("unsupported escape");
                }
                continue;
            }
            out += c;
        }
    }

    Ptr ParseValue() {
        const char c = Peek();
        if (c == '"' || c == '\'') {
            Ptr v = make(TomlValue::String);
            v->str = ParseStringRaw();
            return v;
        }
        if (c == '[') return ParseArray();
        if (c == '{') return ParseInlineTable();
        std::string tok;
        while (!Eof() && !std::isspace((unsigned char)Peek()) && Peek() != ',' && Peek() != ']' && Peek() != '}' &&
               Peek() != '#')
            tok += Get();
        if (tok == "true" || tok == "false") {
            Ptr v = make(TomlValue::Bool);
            v->b = tok == "true";
            return v;
        }
        return ParseNumber(tok);
    }

    Ptr ParseNumber(std::string tok) {
        if (tok.empty()) Fail("expected a value");
        std::string t;
        for (char ch : tok)
            if (ch != '_') t += ch;
        const std::string body = (t[0] == '+' || t[0] == '-') ? t.substr(1) : t;
        const double sign = t[0] == '-' ? -1.0 : 1.0;
        if (body == "inf" || body == "nan") {
            Ptr v = make(TomlValue::Float);
            v->f = body == "inf" ? sign * std::numeric_limits<double>::infinity()
                                 : std::numeric_limits<double>::quiet_NaN();
            return v;
        }
        if (body.size() > 2 && body[0] == '0' && (body[1] == 'x' || body[1] == 'o' || body[1] == 'b')) {
            const int base = body[1] == 'x' ? 16 : (body[1] == 'o' ? 8 : 2);
            char* end = nullptr;
            const long long iv = std::strtoll(body.c_str() + 2, &end, base);
            if (!end || *end) Fail("bad integer '" + tok + "'");
            Ptr v = make(TomlValue::Int);
            v->i = sign < 0 ? -iv : iv;
            return v;
        }
        const bool isfloat = t.find_first_of(".eE") != std::string::npos;
        char* end = nullptr;
        if (isfloat) {
            const double d = std::strtod(t.c_str(), &end);
            if (!end || *end) Fail("bad number '" + tok + "'");
            Ptr v = make(TomlValue::Float);
            v->f = d;
            return v;
        }
        const long long iv = std::strtoll(t.c_str(), &end, 10);
        if (!end || *end) Fail("bad value '" + tok + "'");
        Ptr v = make(TomlValue::Int);
        v->i = iv;
        return v;
    }

    Ptr ParseArray() {
        Expect('[');
        Ptr arr = make(TomlValue::Array);
        for (;;) {
            SkipWsNl();
            if (Peek() == ']') {
                Get();
                return arr;
            }
            arr->array.push_back(ParseValue());
            SkipWsNl();
            if (Peek() == ',') {
                Get();
                continue;
            }
            SkipWsNl();
            Expect(']');
            return arr;
        }
    }

    Ptr ParseInlineTable() {
        Expect('{');
        Ptr t = make(TomlValue::Table);
        SkipWs();
        if (Peek() == '}') {
            Get();
            return t;
        }
        for (;;) {
            std::vector<std::string> key = ParseKey();
            SkipWs();
            Expect('=');
            SkipWs();
            Assign(t.get(), key, ParseValue());
            SkipWs();
            if (Peek() == ',') {
                Get();
                SkipWs();
                continue;
            }
            Expect('}');
            return t;
        }
    }

    std::string_view s_;
    std::string name_;
    size_t pos_ = 0;
    int line_ = 1;
};

std::vector<std::string> SplitPath(std::string_view path) {
    std::vector<std::string> parts;
    std::string cur;
    for (char c : path) {
        if (c == '.') {
            parts.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    parts.push_back(cur);
    return parts;
}

}  // namespace

Deck Deck::FromString(std::string_view toml, std::string sourceName) {
    Deck d;
    d.m_root = Parser(toml, sourceName).Parse();
    d.m_view = d.m_root.get();
    d.m_sourceText.assign(toml);
    d.m_sourceName = std::move(sourceName);
    return d;
}

Deck Deck::FromFile(const std::string& path) {
    std::ifstream f(path, std::ios::in | std::ios::binary);
    if (!f) throw std::runtime_error("Deck: failed to open " + path);
    std::ostringstream ss;
    ss << f.rdbuf();
    return FromString(ss.str(), path);
}

const TomlValue* Deck::Find(std::string_view path) const {
    const TomlValue* t = m_view;
    for (const std::string& k : SplitPath(path)) {
        if (!t || t->kind != TomlValue::Table) return nullptr;
        auto it = t->table.find(k);
        if (it == t->table.end()) return nullptr;
        t = it->second.get();
    }
    return t;
}

bool Deck::Has(std::string_view path) const { return Find(path) != nullptr; }

int Deck::GetInt(std::string_view path, int fallback) const {
    const TomlValue* v = Find(path);
    if (v && v->kind == TomlValue::Int) return (int)v->i;
    if (v && v->kind == TomlValue::Float) return (int)(int64_t)v->f;
    return fallback;
}

double Deck::GetDouble(std::string_view path, double fallback) const {
    const TomlValue* v = Find(path);
    if (v && v->kind == TomlValue::Float) return v->f;
    if (v && v->kind == TomlValue::Int) return (double)v->i;
    return fallback;
}

bool Deck::GetBool(std::string_view path, bool fallback) const {
    const TomlValue* v = Find(path);
    return (v && v->kind == TomlValue::Bool) ? v->b : fallback;
}

std::string Deck::GetString(std::string_view path, std::string_view fallback) const {
    const TomlValue* v = Find(path);
    return (v && v->kind == TomlValue::String) ? v->str : std::string(fallback);
}

std::vector<double> Deck::GetDoubleArray(std::string_view path) const {
    std::vector<double> out;
    const TomlValue* v = Find(path);
    if (v && v->kind == TomlValue::Array)
        for (const auto& e : v->array)
            out.push_back(e->kind == TomlValue::Float ? e->f : (e->kind == TomlValue::Int ? (double)e->i : 0.0));
    return out;
}

std::vector<std::string> Deck::GetStringArray(std::string_view path) const {
    std::vector<std::string> out;
    const TomlValue* v = Find(path);
    if (v && v->kind == TomlValue::Array)
        for (const auto& e : v->array) out.push_back(e->kind == TomlValue::String ? e->str : std::string());
    return out;
}

std::vector<Deck> Deck::GetTables(std::string_view path) const {
    std::vector<Deck> out;
    const TomlValue* v = Find(path);
    if (v && v->kind == TomlValue::Array) {
        for (const auto& e : v->array) {
            if (e->kind != TomlValue::Table) continue;
            Deck sub;
            sub.m_root = m_root;
            sub.m_view = e.get();
            sub.m_sourceName = m_sourceName;
            out.push_back(std::move(sub));
        }
    }
    return out;
}

}  // namespace fw
