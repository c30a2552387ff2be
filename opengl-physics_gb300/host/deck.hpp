// deck.hpp -- TOML input deck with dotted-path access.
//
// Same contract as the reference's fw::Deck (framework/include/framework/
// Deck.hpp:19-55): every knob of a run comes from one TOML file; values are
// read by dotted path ("time.dt"); a missing key returns the caller's
// default; integer and floating-point nodes coerce into each other
// (framework/src/Deck.cpp:80-94); arrays of tables come back as sub-decks.
// Parse errors throw std::runtime_error naming the source and line.
//
// The parser covers the TOML subset the N-body decks use: [tables],
// [[arrays of tables]], dotted and quoted keys, basic and literal strings,
// integers (with _ separators, hex/oct/bin), floats (incl. inf/nan),
// booleans, (multi-line) arrays and inline tables, and # comments.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <string_view>
#include <vector>

namespace fw {

struct TomlValue {
    enum Kind { Table, Array, String, Int, Float, Bool } kind = Table;
    std::map<std::string, std::shared_ptr<TomlValue>> table;
    std::vector<std::shared_ptr<TomlValue>> array;
    std::string str;
    int64_t i = 0;
    double f = 0.0;
    bool b = false;
};

class Deck {
public:
    static Deck FromFile(const std::string& path);
    static Deck FromString(std::string_view toml, std::string sourceName = "<string>");

    bool Has(std::string_view path) const;
    int GetInt(std::string_view path, int fallback) const;
    double GetDouble(std::string_view path, double fallback) const;
    bool GetBool(std::string_view path, bool fallback) const;
    std::string GetString(std::string_view path, std::string_view fallback) const;
    std::vector<double> GetDoubleArray(std::string_view path) const;
    std::vector<std::string> GetStringArray(std::string_view path) const;
    std::vector<Deck> GetTables(std::string_view path) const;

    // The parsed table this deck views (the whole file, or one sub-table).
    const TomlValue& Root() const { return *m_view; }
    const std::string& SourceText() const { return m_sourceText; }
    const std::string& SourceName() const { return m_sourceName; }

private:
    const TomlValue* Find(std::string_view path) const;

    std::shared_ptr<TomlValue> m_root;
    const TomlValue* m_view = nullptr;
    std::string m_sourceText;
    std::string m_sourceName;
};

}  // namespace fw
