// json_text.cpp -- strict JSON parser and deterministic writer (conventions in json_text.h).
#include "json_text.h"

#include <charconv>
#include <cmath>
#include <cstring>
#include <string>
#include <unordered_set>

namespace rcwa_gb300 {
namespace jtext {

bool Value::to_int(int& out) const {
    if (kind != Kind::Number) return false;
    if (!(number >= -2147483648.0 && number <= 2147483647.0) || number != std::floor(number)) return false;
    out = static_cast<int>(number);
    return true;
}

namespace {

// bytes of the UTF-8 character starting at s[0] (>= 0x80), 0 when malformed: overlong forms, surrogates
// and code points above U+10FFFF are rejected
std::size_t utf8_size(const unsigned char* s, std::size_t avail) {
    const auto cont = [&](std::size_t k) { return k < avail && (s[k] & 0xC0) == 0x80; };
    const unsigned char b = s[0];
    if (b >= 0xC2 && b <= 0xDF) return cont(1) ? 2 : 0;
    if (b >= 0xE0 && b <= 0xEF) {
        if (!cont(1) || !cont(2)) return 0;
        if ((b == 0xE0 && s[1] < 0xA0) || (b == 0xED && s[1] > 0x9F)) return 0;
        return 3;
    }
    if (b >= 0xF0 && b <= 0xF4) {
        if (!cont(1) || !cont(2) || !cont(3)) return 0;
        if ((b == 0xF0 && s[1] < 0x90) || (b == 0xF4 && s[1] > 0x8F)) return 0;
        return 4;
    }
    return 0;
}

void put_utf8(std::string& out, unsigned long cp) {
    if (cp < 0x80) {
        out.push_back(static_cast<char>(cp));
    } else if (cp < 0x800) {
        out.push_back(static_cast<char>(0xC0 | (cp >> 6)));
        out.push_back(static_cast<char>(0x80 | (cp & 0x3F)));
    } else if (cp < 0x10000) {
        out.push_back(static_cast<char>(0xE0 | (cp >> 12)));
        out.push_back(static_cast<char>(0x80 | ((cp >> 6) & 0x3F)));
        out.push_back(static_cast<char>(0x80 | (cp & 0x3F)));
    } else {
        out.push_back(static_cast<char>(0xF0 | (cp >> 18)));
        out.push_back(static_cast<char>(0x80 | ((cp >> 12) & 0x3F)));
        out.push_back(static_cast<char>(0x80 | ((cp >> 6) & 0x3F)));
        out.push_back(static_cast<char>(0x80 | (cp & 0x3F)));
    }
}

class Reader {
public:
    Reader(const std::string& s, int max_depth)
        : p_(reinterpret_cast<const unsigned char*>(s.data())), n_(s.size()), max_depth_(max_depth) {}

    Value document() {
        if (n_ >= 3 && p_[0] == 0xEF && p_[1] == 0xBB && p_[2] == 0xBF) i_ = 3;
        space();
        Value v = value(0);
        space();
        if (i_ < n_) fail("unexpected " + shown(i_) + " after the JSON value", i_);
        return v;
    }

private:
    [[noreturn]] void fail(const std::string& why, std::size_t at) const {
        ParseError e;
        e.reason = why;
        e.offset = at;
        std::size_t line = 1, col = 1;
        for (std::size_t k = 0; k < at && k < n_; ++k) {
            if (p_[k] == '\n') {
                ++line;
                col = 1;
            } else if ((p_[k] & 0xC0) != 0x80) {
                ++col;
            }
        }
        e.line = line;
        e.column = col;
        throw e;
    }
    std::string shown(std::size_t at) const {
        const unsigned char c = p_[at];
        if (c >= 0x20 && c < 0x7F) return std::string("character '") + static_cast<char>(c) + "'";
        char buf[16];
        std::snprintf(buf, sizeof buf, "byte 0x%02X", c);
        return buf;
    }
    void space() {
        while (i_ < n_ && (p_[i_] == ' ' || p_[i_] == '\t' || p_[i_] == '\n' || p_[i_] == '\r')) ++i_;
    }
    static bool digit(unsigned char c) { return c >= '0' && c <= '9'; }

    Value value(int depth) {
        if (i_ >= n_) fail("unexpected end of input", i_);
        const unsigned char c = p_[i_];
        if (c == '{') return object(depth);
        if (c == '[') return array(depth);
        if (c == '"') {
            Value v;
            v.kind = Kind::String;
            v.text = string();
            return v;
        }
        if (c == 't' || c == 'f' || c == 'n') return literal();
        if (c == '-' || digit(c)) return number();
        fail("unexpected " + shown(i_), i_);
    }

    Value literal() {
        Value v;
        const auto match = [&](const char* word) {
            const std::size_t len = std::strlen(word);
            return n_ - i_ >= len && std::memcmp(p_ + i_, word, len) == 0;
        };
        if (match("true")) {
            v.kind = Kind::Bool;
            v.boolean = true;
            i_ += 4;
        } else if (match("false")) {
            v.kind = Kind::Bool;
            i_ += 5;
        } else if (match("null")) {
            i_ += 4;
        } else {
            fail("invalid literal (expected true, false or null)", i_);
        }
        return v;
    }

    Value number() {
        const std::size_t start = i_;
        bool plain = true;
        if (p_[i_] == '-') {
            ++i_;
            if (i_ >= n_ || !digit(p_[i_])) fail("a digit must follow the minus sign", i_);
        }
        if (p_[i_] == '0') {
            ++i_;
            if (i_ < n_ && digit(p_[i_])) fail("leading zeros are not allowed in a number", start);
        } else {
            while (i_ < n_ && digit(p_[i_])) ++i_;
        }
        if (i_ < n_ && p_[i_] == '.') {
            plain = false;
            ++i_;
            if (i_ >= n_ || !digit(p_[i_])) fail("a digit must follow the decimal point", i_);
            while (i_ < n_ && digit(p_[i_])) ++i_;
        }
        if (i_ < n_ && (p_[i_] == 'e' || p_[i_] == 'E')) {
            plain = false;
            ++i_;
            if (i_ < n_ && (p_[i_] == '+' || p_[i_] == '-')) ++i_;
            if (i_ >= n_ || !digit(p_[i_])) fail("a digit must follow the exponent mark", i_);
            while (i_ < n_ && digit(p_[i_])) ++i_;
        }
        double x = 0.0;
        const char* b = reinterpret_cast<const char*>(p_ + start);
        const char* e = reinterpret_cast<const char*>(p_ + i_);
        const std::from_chars_result r = std::from_chars(b, e, x);
        if (r.ec != std::errc() || r.ptr != e || !std::isfinite(x)) fail("number is outside the range of double", start);
        Value v;
        v.kind = Kind::Number;
        v.number = x;
        v.integer = plain && std::fabs(x) <= 9007199254740991.0;
        return v;
    }

    unsigned hex4(std::size_t escape) {
        if (n_ - i_ < 4) fail("\\u must be followed by four hexadecimal digits", escape);
        unsigned v = 0;
        for (int k = 0; k < 4; ++k) {
            const unsigned char c = p_[i_ + k];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= c - '0';
            else if (c >= 'a' && c <= 'f') v |= c - 'a' + 10;
            else if (c >= 'A' && c <= 'F') v |= c - 'A' + 10;
            else fail("\\u must be followed by four hexadecimal digits", escape);
        }
        i_ += 4;
        return v;
    }

    std::string string() {
        const std::size_t opened = i_++;
        std::string out;
        for (;;) {
            if (i_ >= n_) fail("unterminated string", opened);
            const unsigned char c = p_[i_];
            if (c == '"') {
                ++i_;
                return out;
            }
            if (c < 0x20) fail("control character in a string (it must be escaped)", i_);
            if (c >= 0x80) {
                const std::size_t len = utf8_size(p_ + i_, n_ - i_);
                if (len == 0) fail("invalid UTF-8 in a string", i_);
                out.append(reinterpret_cast<const char*>(p_ + i_), len);
                i_ += len;
                continue;
            }
            if (c != '\\') {
                out.push_back(static_cast<char>(c));
                ++i_;
                continue;
            }
            const std::size_t escape = i_++;
            if (i_ >= n_) fail("unterminated string", opened);
            const unsigned char e = p_[i_++];
            switch (e) {
                case '"': out.push_back('"'); break;
                case '\\': out.push_back('\\'); break;
                case '/': out.push_back('/'); break;
                case 'b': out.push_back('\b'); break;
                case 'f': out.push_back('\f'); break;
                case 'n': out.push_back('\n'); break;
                case 'r': out.push_back('\r'); break;
                case 't': out.push_back('\t'); break;
                case 'u': {
                    unsigned long cp = hex4(escape);
                    if (cp >= 0xDC00 && cp <= 0xDFFF) fail("unpaired surrogate in a \\u escape", escape);
                    if (cp >= 0xD800 && cp <= 0xDBFF) {
                        if (n_ - i_ < 2 || p_[i_] != '\\' || p_[i_ + 1] != 'u') fail("unpaired surrogate in a \\u escape", escape);
                        i_ += 2;
                        const unsigned long low = hex4(escape);
                        if (low < 0xDC00 || low > 0xDFFF) fail("unpaired surrogate in a \\u escape", escape);
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (low - 0xDC00);
                    }
                    put_utf8(out, cp);
                    break;
                }
                default: fail("invalid escape sequence in a string", escape);
            }
        }
    }

    Value array(int depth) {
        const std::size_t opened = i_;
        if (depth >= max_depth_) fail("arrays and objects are nested too deeply", opened);
        ++i_;
        Value v;
        v.kind = Kind::Array;
        space();
        if (i_ < n_ && p_[i_] == ']') {
            ++i_;
            return v;
        }
        for (;;) {
            space();
            v.items.push_back(value(depth + 1));
            space();
            if (i_ >= n_) fail("unexpected end of input inside an array", i_);
            if (p_[i_] == ']') {
                ++i_;
                return v;
            }
            if (p_[i_] != ',') fail("expected ',' or ']' in an array, found " + shown(i_), i_);
            ++i_;
        }
    }

    Value object(int depth) {
        const std::size_t opened = i_;
        if (depth >= max_depth_) fail("arrays and objects are nested too deeply", opened);
        ++i_;
        Value v;
        v.kind = Kind::Object;
        std::vector<std::size_t> where;
        space();
        if (i_ < n_ && p_[i_] == '}') {
            ++i_;
            return v;
        }
        for (;;) {
            space();
            if (i_ >= n_) fail("unexpected end of input inside an object", i_);
            if (p_[i_] != '"') fail("expected a string key in an object, found " + shown(i_), i_);
            where.push_back(i_);
            v.keys.push_back(string());
            space();
            if (i_ >= n_) fail("unexpected end of input inside an object", i_);
            if (p_[i_] != ':') fail("expected ':' after an object key, found " + shown(i_), i_);
            ++i_;
            space();
            v.items.push_back(value(depth + 1));
            space();
            if (i_ >= n_) fail("unexpected end of input inside an object", i_);
            if (p_[i_] == '}') {
                ++i_;
                break;
            }
            if (p_[i_] != ',') fail("expected ',' or '}' in an object, found " + shown(i_), i_);
            ++i_;
        }
        // a repeated key is reported at its first repetition
        std::unordered_set<std::string> seen;
        for (std::size_t k = 0; k < v.keys.size(); ++k)
            if (!seen.insert(v.keys[k]).second) fail("duplicate key in an object", where[k]);
        return v;
    }

    const unsigned char* p_;
    std::size_t n_, i_ = 0;
    int max_depth_;
};

}  // namespace

Value parse(const std::string& text, int max_depth) { return Reader(text, max_depth).document(); }

// ------------------------------------------------------------------ writing

void append_double(std::string& out, double x) {
    if (!std::isfinite(x)) {
        out += "null";
        return;
    }
    std::string best;
    for (int digits = 15; digits <= 17; ++digits) {
        char buf[64];
        const std::to_chars_result r = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::general, digits);
        std::string s(buf, r.ptr);
        // normalise: exponent sign always present with at least two digits; ".0" when neither '.' nor exponent
        const std::size_t e = s.find('e');
        if (e != std::string::npos) {
            std::string mant = s.substr(0, e), ex = s.substr(e + 1);
            char sign = '+';
            if (!ex.empty() && (ex[0] == '+' || ex[0] == '-')) {
                sign = ex[0];
                ex.erase(0, 1);
            }
            while (ex.size() > 2 && ex[0] == '0') ex.erase(0, 1);
            if (ex.size() < 2) ex.insert(0, "0");
            s = mant + "e" + sign + ex;
        } else if (s.find('.') == std::string::npos) {
            s += ".0";
        }
        best = s;
        double back = 0.0;
        const std::from_chars_result q = std::from_chars(s.data(), s.data() + s.size(), back);
        if (q.ec == std::errc() && back == x) break;
    }
    out += best;
}

void append_string(std::string& out, const std::string& s) {
    static const char hex[] = "0123456789abcdef";
    out.push_back('"');
    const auto* p = reinterpret_cast<const unsigned char*>(s.data());
    std::size_t i = 0;
    while (i < s.size()) {
        const unsigned char c = p[i];
        if (c == '"') {
            out += "\\\"";
        } else if (c == '\\') {
            out += "\\\\";
        } else if (c < 0x20) {
            switch (c) {
                case '\b': out += "\\b"; break;
                case '\f': out += "\\f"; break;
                case '\n': out += "\\n"; break;
                case '\r': out += "\\r"; break;
                case '\t': out += "\\t"; break;
                default:
                    out += "\\u00";
                    out.push_back(hex[c >> 4]);
                    out.push_back(hex[c & 15]);
            }
        } else if (c < 0x80) {
            out.push_back(static_cast<char>(c));
        } else {
            const std::size_t len = utf8_size(p + i, s.size() - i);
            if (len == 0) {
                out += "\xEF\xBF\xBD";  // U+FFFD for a malformed byte
            } else {
                out.append(s, i, len);
                i += len;
                continue;
            }
        }
        ++i;
    }
    out.push_back('"');
}

void Writer::separate() {
    Frame& f = stack_.back();
    if (!f.empty) out_.push_back(',');
    if (!f.flat) {
        out_.push_back('\n');
        out_.append(stack_.size() * static_cast<std::size_t>(indent_), ' ');
    } else if (!f.empty) {
        out_.push_back(' ');
    }
    f.empty = false;
}
void Writer::before_value() {
    if (stack_.empty()) return;
    if (stack_.back().object) {
        keyed_ = false;
        return;
    }
    separate();
}
void Writer::key(const std::string& name) {
    separate();
    append_string(out_, name);
    out_ += ": ";
    keyed_ = true;
}
void Writer::null() {
    before_value();
    out_ += "null";
}
void Writer::value(bool b) {
    before_value();
    out_ += b ? "true" : "false";
}
void Writer::value_integer(long long x) {
    before_value();
    out_ += std::to_string(x);
}
void Writer::value(double x) {
    before_value();
    append_double(out_, x);
}
void Writer::value(const std::string& s) {
    before_value();
    append_string(out_, s);
}
void Writer::open(char bracket, bool object, bool one_line) {
    before_value();
    const bool flat = indent_ < 0 || one_line || (!stack_.empty() && stack_.back().flat);
    stack_.push_back(Frame{object, flat, true});
    out_.push_back(bracket);
}
void Writer::close(char bracket) {
    const Frame f = stack_.back();
    stack_.pop_back();
    if (!f.flat && !f.empty) {
        out_.push_back('\n');
        out_.append(stack_.size() * static_cast<std::size_t>(indent_), ' ');
    }
    out_.push_back(bracket);
}

}  // namespace jtext
}  // namespace rcwa_gb300
