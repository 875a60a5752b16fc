// toml.cpp -- recursive-descent reader for the TOML subset in toml.hpp.
#include "toml.hpp"

#include <cmath>
#include <cstdlib>
#include <limits>

namespace mdg_host {
namespace toml {

double Value::number() const {
    if (kind == INT) return (double)i;
    if (kind == FLOAT) return f;
    throw Error("expected a number");
}
const Table& Value::table() const {
    if (kind != TABLE) throw Error("expected a table");
    return *t;
}
const Array& Value::array() const {
    if (kind != ARRAY) throw Error("expected an array");
    return *a;
}
const std::string& Value::str() const {
    if (kind != STRING) throw Error("expected a string");
    return s;
}
bool Value::boolean() const {
    if (kind != BOOL) throw Error("expected a boolean");
    return b;
}
int64_t Value::integer() const {
    if (kind == INT) return i;
    if (kind == FLOAT && std::floor(f) == f && std::fabs(f) < 9.0e15) return (int64_t)f;
    throw Error("expected an integer");
}

const Value* find(const Table& t, const std::string& key) {
    auto it = t.find(key);
    return it == t.end() ? nullptr : &it->second;
}

namespace {

Value make_table() {
    Value v;
    v.kind = Value::TABLE;
    v.t = std::make_shared<Table>();
    return v;
}

Value make_array() {
    Value v;
    v.kind = Value::ARRAY;
    v.a = std::make_shared<Array>();
    return v;
}

void append_utf8(std::string& out, uint32_t cp) {
    if (cp < 0x80) {
        out += (char)cp;
    } else if (cp < 0x800) {
        out += (char)(0xC0 | (cp >> 6));
        out += (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
        out += (char)(0xE0 | (cp >> 12));
        out += (char)(0x80 | ((cp >> 6) & 0x3F));
        out += (char)(0x80 | (cp & 0x3F));
    } else {
        out += (char)(0xF0 | (cp >> 18));
        out += (char)(0x80 | ((cp >> 12) & 0x3F));
        out += (char)(0x80 | ((cp >> 6) & 0x3F));
        out += (char)(0x80 | (cp & 0x3F));
    }
}

class Parser {
public:
    explicit Parser(const std::string& text) : s_(text) {}

    Table run() {
        Table* cur = &root_;
        while (true) {
            skip_ws();
            if (eof()) break;
            const char c = peek();
            if (c == '#') {
                skip_comment();
                continue;
            }
            if (c == '\n' || c == '\r') {
                newline();
                continue;
            }
            if (c == '[') {
                cur = header();
            } else {
                key_value(*cur);
            }
            end_of_line();
        }
        return root_;
    }

private:
    const std::string& s_;
    size_t p_ = 0;
    int line_ = 1;
    Table root_;

    [[noreturn]] void fail(const std::string& m) const { throw Error("line " + std::to_string(line_) + ": " + m); }
    bool eof() const { return p_ >= s_.size(); }
    char peek(size_t k = 0) const { return p_ + k < s_.size() ? s_[p_ + k] : '\0'; }
    char get() {
        if (eof()) fail("unexpected end of input");
        return s_[p_++];
    }
    void skip_ws() {
        while (!eof() && (peek() == ' ' || peek() == '\t')) p_++;
    }
    void skip_comment() {
        while (!eof() && peek() != '\n') p_++;
    }
    void newline() {
        if (peek() == '\r') p_++;
        if (peek() == '\n') {
            p_++;
            line_++;
        }
    }
    // whitespace, newlines and comments (inside arrays)
    void skip_all() {
        while (!eof()) {
            const char c = peek();
            if (c == ' ' || c == '\t') p_++;
            else if (c == '\n' || c == '\r') newline();
            else if (c == '#') skip_comment();
            else break;
        }
    }
    void end_of_line() {
        skip_ws();
        if (peek() == '#') skip_comment();
        if (eof()) return;
        if (peek() != '\n' && peek() != '\r') fail("expected the end of the line");
        newline();
    }

    static bool bare(char c) {
        return (c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || (c >= '0' && c <= '9') || c == '_' || c == '-';
    }

    std::string key_part() {
        skip_ws();
        const char c = peek();
        if (c == '"' || c == '\'') return string_value().s;
        std::string k;
        while (!eof() && bare(peek())) k += get();
        if (k.empty()) fail("expected a key");
        return k;
    }

    std::vector<std::string> key() {
        std::vector<std::string> path{key_part()};
        skip_ws();
        while (peek() == '.') {
            p_++;
            path.push_back(key_part());
            skip_ws();
        }
        return path;
    }

    // Walk a header path: missing tables are created; an array of tables
    // continues in its last element.
    Table* walk(Table* base, const std::vector<std::string>& path, size_t n) {
        for (size_t k = 0; k < n; k++) {
            auto it = base->find(path[k]);
            if (it == base->end()) it = base->emplace(path[k], make_table()).first;
            Value& v = it->second;
            if (v.kind == Value::TABLE) {
                base = v.t.get();
            } else if (v.kind == Value::ARRAY && !v.a->empty() && v.a->back().kind == Value::TABLE) {
                base = v.a->back().t.get();
            } else {
                fail("key '" + path[k] + "' is not a table");
            }
        }
        return base;
    }

    Table* header() {
        p_++;  // '['
        const bool arr = peek() == '[';
        if (arr) p_++;
        const std::vector<std::string> path = key();
        skip_ws();
        if (get() != ']') fail("expected ']'");
        if (arr && get() != ']') fail("expected ']]'");
        Table* parent = walk(&root_, path, path.size() - 1);
        const std::string& last = path.back();
        auto it = parent->find(last);
        if (arr) {
            if (it == parent->end()) it = parent->emplace(last, make_array()).first;
            if (it->second.kind != Value::ARRAY) fail("key '" + last + "' is not an array of tables");
            it->second.a->push_back(make_table());
            return it->second.a->back().t.get();
        }
        if (it == parent->end()) it = parent->emplace(last, make_table()).first;
        if (it->second.kind != Value::TABLE) fail("key '" + last + "' is not a table");
        return it->second.t.get();
    }

    void key_value(Table& t) {
        const std::vector<std::string> path = key();
        skip_ws();
        if (get() != '=') fail("expected '='");
        skip_ws();
        Value v = value();
        Table* dst = walk(&t, path, path.size() - 1);
        if (dst->count(path.back())) fail("duplicate key '" + path.back() + "'");
        dst->emplace(path.back(), std::move(v));
    }

    Value value() {
        const char c = peek();
        if (c == '"' || c == '\'') return string_value();
        if (c == '[') return array_value();
        if (c == '{') return inline_table();
        return scalar();
    }

    Value string_value() {
        Value v;
        v.kind = Value::STRING;
        const char q = get();
        const bool multi = peek() == q && peek(1) == q;
        if (multi) {
            p_ += 2;
            if (peek() == '\r') p_++;
            if (peek() == '\n') {  // a newline right after the opening quotes is trimmed
                p_++;
                line_++;
            }
        }
        while (true) {
            if (eof()) fail("unterminated string");
            const char c = get();
            if (c == q) {
                if (!multi) break;
                if (peek() == q && peek(1) == q) {
                    p_ += 2;
                    break;
                }
                v.s += c;
                continue;
            }
            if (c == '\n') {
                if (!multi) fail("newline in a string");
                line_++;
                v.s += c;
                continue;
            }
            if (c == '\\' && q == '"') {
                const char e = get();
                switch (e) {
                    case 'b': v.s += '\b'; break;
                    case 't': v.s += '\t'; break;
                    case 'n': v.s += '\n'; break;
                    case 'f': v.s += '\f'; break;
                    case 'r': v.s += '\r'; break;
                    case '"': v.s += '"'; break;
                    case '\\': v.s += '\\'; break;
                    case 'u':
                    case 'U': {
                        const int nd = e == 'u' ? 4 : 8;
                        std::string h;
                        for (int k = 0; k < nd; k++) h += get();
                        char* end = nullptr;
                        const unsigned long cp = std::strtoul(h.c_str(), &end, 16);
                        if (*end) fail("bad unicode escape");
                        append_utf8(v.s, (uint32_t)cp);
                        break;
                    }
                    case '\n':
                    case '\r':
                        if (!multi) fail("bad escape");
                        newline();  // line-ending backslash: trim the newline and following whitespace
                        skip_all();
                        break;
                    default: fail(std::string("bad escape \\") + e);
                }
                continue;
            }
            v.s += c;
        }
        return v;
    }

    Value array_value() {
        p_++;  // '['
        Value v = make_array();
        skip_all();
        while (peek() != ']') {
            v.a->push_back(value());
            skip_all();
            if (peek() == ',') {
                p_++;
                skip_all();
            } else if (peek() != ']') {
                fail("expected ',' or ']' in an array");
            }
        }
        p_++;  // ']'
        return v;
    }

    Value inline_table() {
        p_++;  // '{'
        Value v = make_table();
        skip_ws();
        if (peek() == '}') {
            p_++;
            return v;
        }
        while (true) {
            key_value(*v.t);
            skip_ws();
            const char c = get();
            if (c == '}') break;
            if (c != ',') fail("expected ',' or '}' in an inline table");
        }
        return v;
    }

    Value scalar() {
        std::string tok;
        while (!eof()) {
            const char c = peek();
            if (c == ',' || c == ']' || c == '}' || c == ' ' || c == '\t' || c == '#' || c == '\n' || c == '\r') break;
            tok += get();
        }
        if (tok.empty()) fail("expected a value");
        Value v;
        if (tok == "true" || tok == "false") {
            v.kind = Value::BOOL;
            v.b = tok == "true";
            return v;
        }
        std::string t;
        for (char c : tok)
            if (c != '_') t += c;
        const std::string body = (t[0] == '+' || t[0] == '-') ? t.substr(1) : t;
        const double sign = t[0] == '-' ? -1.0 : 1.0;
        if (body == "inf" || body == "nan") {
            v.kind = Value::FLOAT;
            v.f = body == "inf" ? sign * std::numeric_limits<double>::infinity()
                                : std::numeric_limits<double>::quiet_NaN();
            return v;
        }
        char* end = nullptr;
        if (body.size() > 2 && body[0] == '0' && (body[1] == 'x' || body[1] == 'o' || body[1] == 'b')) {
            const int base = body[1] == 'x' ? 16 : (body[1] == 'o' ? 8 : 2);
            const long long x = std::strtoll(body.c_str() + 2, &end, base);
            if (*end) fail("bad number '" + tok + "'");
            v.kind = Value::INT;
            v.i = x;
            return v;
        }
        const bool is_float = t.find_first_of(".eE") != std::string::npos;
        if (is_float) {
            const double x = std::strtod(t.c_str(), &end);
            if (*end) fail("bad number '" + tok + "'");
            v.kind = Value::FLOAT;
            v.f = x;
        } else {
            const long long x = std::strtoll(t.c_str(), &end, 10);
            if (*end) fail("bad value '" + tok + "'");
            v.kind = Value::INT;
            v.i = x;
        }
        return v;
    }
};

}  // namespace

Table parse(const std::string& text) { return Parser(text).run(); }

}  // namespace toml
}  // namespace mdg_host
