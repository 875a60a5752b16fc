// toml.hpp -- the subset of TOML 1.0 that MDDEM configs use: tables, dotted
// table headers, arrays of tables, dotted keys, basic and literal strings,
// integers, floats (incl. inf / nan and exponents), booleans, arrays (also
// across lines) and inline tables.  Dates are not supported.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace mdg_host {
namespace toml {

struct Value;
using Table = std::map<std::string, Value>;
using Array = std::vector<Value>;

struct Value {
    enum Kind { NONE, BOOL, INT, FLOAT, STRING, ARRAY, TABLE } kind = NONE;
    bool b = false;
    int64_t i = 0;
    double f = 0.0;
    std::string s;
    std::shared_ptr<Array> a;
    std::shared_ptr<Table> t;

    bool is_number() const { return kind == INT || kind == FLOAT; }
    double number() const;                 // INT or FLOAT, else throws
    const Table& table() const;            // TABLE, else throws
    const Array& array() const;            // ARRAY, else throws
    const std::string& str() const;        // STRING, else throws
    bool boolean() const;                  // BOOL, else throws
    int64_t integer() const;               // INT (or an integral FLOAT), else throws
};

struct Error : std::runtime_error {
    explicit Error(const std::string& m) : std::runtime_error(m) {}
};

// Parse a document; throws Error with the line number on malformed input.
Table parse(const std::string& text);

// Lookups that return nullptr when a key is absent.
const Value* find(const Table& t, const std::string& key);

}  // namespace toml
}  // namespace mdg_host
