// json_text.h -- the JSON text layer of the request front end: a value tree, a strict parser and a
// deterministic writer with the conventions of the StableRCWA wire format (include/stablercwa/json.hpp):
//   parse   RFC 8259 only (no comments, NaN, trailing commas, leading zeros); numbers are correctly rounded
//           doubles and out-of-range numbers are errors; strings are validated UTF-8 with \u escapes and
//           surrogate pairs; duplicate keys and nesting deeper than 128 levels are errors; a leading BOM is
//           skipped. Errors carry the byte offset and the 1-based line and column (column in characters).
//   write   the shortest of 15, 16, 17 significant digits that reads back to the same double, integers
//           without a decimal point, other numbers always with '.' or an exponent (e+NN / e-NN, at least two
//           digits), NaN and infinities as null; ", " and ": " separators on one line, or one item per line
//           with an indent for objects and for arrays that hold objects.
#pragma once

#include <cstddef>
#include <string>
#include <vector>

namespace rcwa_gb300 {
namespace jtext {

enum class Kind { Null, Bool, Number, String, Array, Object };

struct ParseError {
    std::string reason;
    std::size_t offset = 0, line = 1, column = 1;
};

class Value {
public:
    Kind kind = Kind::Null;
    bool boolean = false;
    bool integer = false;  // written without '.' or exponent and |x| < 2^53
    double number = 0.0;
    std::string text;
    std::vector<Value> items;       // array elements, or object values in key order
    std::vector<std::string> keys;  // object keys

    bool is_number() const { return kind == Kind::Number; }
    bool is_string() const { return kind == Kind::String; }
    bool is_bool() const { return kind == Kind::Bool; }
    bool is_array() const { return kind == Kind::Array; }
    bool is_object() const { return kind == Kind::Object; }
    std::size_t size() const { return items.size(); }
    const Value& at(std::size_t i) const { return items.at(i); }
    const Value* find(const std::string& key) const {
        for (std::size_t i = 0; i < keys.size(); ++i)
            if (keys[i] == key) return &items[i];
        return nullptr;
    }
    bool contains(const std::string& key) const { return find(key) != nullptr; }
    // an integral number within int range (20, 20.0 and 2e1 all count)
    bool to_int(int& out) const;
};

// Throws ParseError.
Value parse(const std::string& text, int max_depth = 128);

class Writer {
public:
    explicit Writer(int indent = -1) : indent_(indent > 16 ? 16 : indent) {}
    void begin_object(bool one_line = false) { open('{', true, one_line); }
    void end_object() { close('}'); }
    void begin_array(bool one_line = false) { open('[', false, one_line); }
    void end_array() { close(']'); }
    void key(const std::string& name);
    void null();
    void value(bool b);
    void value(int x) { value_integer(x); }
    void value(long long x) { value_integer(x); }
    void value(double x);
    void value(const std::string& s);
    void value(const char* s) { value(std::string(s)); }
    void complex(double re, double im) {
        begin_array(true);
        value(re);
        value(im);
        end_array();
    }
    std::string take() { return std::move(out_); }

private:
    struct Frame {
        bool object, flat, empty;
    };
    void value_integer(long long x);
    void before_value();
    void separate();
    void open(char bracket, bool object, bool one_line);
    void close(char bracket);
    int indent_;
    std::string out_;
    std::vector<Frame> stack_;
    bool keyed_ = false;
};

void append_double(std::string& out, double x);
void append_string(std::string& out, const std::string& s);

}  // namespace jtext
}  // namespace rcwa_gb300
