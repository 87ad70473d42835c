// Words of a line, for the text formats the host layer reads (.scene, OBJ, MTL).
//
// A line is split into its blank-separated words and read front to back by a
// cursor. A value is always a whole word: a number is a word made only of
// digits, signs, a decimal point and an exponent that converts completely to
// a finite double (so "inf", "nan" and hexadecimal forms are not numbers, as
// they are not for a C++ stream); an integer is a number without a point or
// an exponent that fits an int. Readers that fail leave the cursor where it
// was, so a caller can test for an optional value.
#pragma once

#include <algorithm>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "host_math.h"

namespace mypbr_host {

inline bool word_is_number(const std::string& s, double& x) {
    if (s.empty() || s.size() > 96)
        return false;
    for (char c : s)
        if (!((c >= '0' && c <= '9') || c == '+' || c == '-' || c == '.' || c == 'e' || c == 'E'))
            return false;
    errno = 0;
    char* end = nullptr;
    double v = std::strtod(s.c_str(), &end);
    if (end != s.c_str() + s.size() || !std::isfinite(v) || errno == ERANGE)
        return false;
    x = v;
    return true;
}

inline bool word_is_integer(const std::string& s, int& x) {
    size_t k = (!s.empty() && (s[0] == '+' || s[0] == '-')) ? 1 : 0;
    if (k == s.size() || s.size() - k > 10)
        return false;
    long long v = 0;
    for (size_t i = k; i < s.size(); i++) {
        if (s[i] < '0' || s[i] > '9')
            return false;
        v = v * 10 + (s[i] - '0');
    }
    if (s[0] == '-')
        v = -v;
    if (v < INT_MIN || v > INT_MAX)
        return false;
    x = int(v);
    return true;
}

// A closed or open interval a number must lie in.
struct Bound {
    double lo = -kInf, hi = kInf;
    bool lo_open = false, hi_open = false;
    bool holds(double x) const {
        return (lo_open ? x > lo : x >= lo) && (hi_open ? x < hi : x <= hi);
    }
};
inline Bound any_value() { return Bound{}; }
inline Bound positive() { return Bound{0, kInf, true, false}; }
inline Bound non_negative() { return Bound{0, kInf, false, false}; }
inline Bound between(double lo, double hi, bool lo_open, bool hi_open) { return Bound{lo, hi, lo_open, hi_open}; }

class Words {
  public:
    Words() = default;
    explicit Words(const std::string& text) {
        size_t i = 0, n = text.size();
        while (i < n) {
            while (i < n && is_blank(text[i]))
                i++;
            size_t start = i;
            while (i < n && !is_blank(text[i]))
                i++;
            if (i > start)
                words_.push_back(text.substr(start, i - start));
        }
    }

    bool more() const { return at_ < words_.size(); }
    size_t left() const { return words_.size() - at_; }
    const std::string& peek(size_t ahead = 0) const {
        static const std::string none;
        return at_ + ahead < words_.size() ? words_[at_ + ahead] : none;
    }
    void skip(size_t n = 1) { at_ = std::min(words_.size(), at_ + n); }

    bool word(std::string& out) {
        if (!more())
            return false;
        out = words_[at_++];
        return true;
    }
    bool next_is_number() const {
        double x;
        return more() && word_is_number(words_[at_], x);
    }
    bool number(double& x, const Bound& b = Bound{}) {
        double v;
        if (!more() || !word_is_number(words_[at_], v) || !b.holds(v))
            return false;
        x = v;
        at_++;
        return true;
    }
    bool integer(int& x) {
        int v;
        if (!more() || !word_is_integer(words_[at_], v))
            return false;
        x = v;
        at_++;
        return true;
    }
    // Three numbers, each within b; on failure nothing is consumed.
    bool triple(V3& v, const Bound& b = Bound{}) {
        size_t mark = at_;
        V3 t;
        if (number(t.x, b) && number(t.y, b) && number(t.z, b)) {
            v = t;
            return true;
        }
        at_ = mark;
        return false;
    }
    bool triple(double out[3], const Bound& b = Bound{}) {
        V3 v;
        if (!triple(v, b))
            return false;
        out[0] = v.x;
        out[1] = v.y;
        out[2] = v.z;
        return true;
    }
    // The words not read yet, joined by single blanks.
    std::string rest() const {
        std::string s;
        for (size_t k = at_; k < words_.size(); k++)
            s += (k > at_ ? " " : "") + words_[k];
        return s;
    }

  private:
    static bool is_blank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f'; }
    std::vector<std::string> words_;
    size_t at_ = 0;
};

}  // namespace mypbr_host
