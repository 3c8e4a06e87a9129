/* Stand-in for boost::format as the reference uses it: a printf-style
 * format string fed with operator% and turned into text with str() or
 * operator<<.  Only the conversions the reference needs (%d %f %X and
 * flags/width/precision) are handled, by handing each directive to
 * snprintf. */
#ifndef ORACLE_BOOST_FORMAT_SHIM
#define ORACLE_BOOST_FORMAT_SHIM
#include <string>
#include <cstdio>
#include <ostream>
#include <type_traits>
namespace boost {
class format {
public:
    explicit format(const std::string &f) : fmt_(f), pos_(0) { advance(); }
    template <class T> format &operator%(const T &v) {
        size_t start = pos_;
        size_t end = start + 1;
        while (end < fmt_.size() && std::string("diouxXeEfFgGcs").find(fmt_[end]) == std::string::npos) ++end;
        std::string spec = fmt_.substr(start, end - start + 1);
        char buf[256];
        emit(buf, sizeof(buf), spec, v);
        out_ += buf;
        pos_ = end + 1;
        advance();
        return *this;
    }
    std::string str() const { return out_; }
private:
    void advance() {
        while (pos_ < fmt_.size()) {
            if (fmt_[pos_] == '%') {
                if (pos_ + 1 < fmt_.size() && fmt_[pos_ + 1] == '%') { out_ += '%'; pos_ += 2; continue; }
                return;
            }
            out_ += fmt_[pos_++];
        }
    }
    template <class T>
    static void emit(char *b, size_t n, const std::string &spec, const T &v) {
        if (std::is_floating_point<T>::value) std::snprintf(b, n, spec.c_str(), (double)v);
        else std::snprintf(b, n, spec.c_str(), (long long)v);
    }
    static void emit(char *b, size_t n, const std::string &, const std::string &v) { std::snprintf(b, n, "%s", v.c_str()); }
    static void emit(char *b, size_t n, const std::string &, const char *v) { std::snprintf(b, n, "%s", v); }
    std::string fmt_;
    size_t pos_;
    std::string out_;
};
inline std::string str(const format &f) { return f.str(); }
inline std::ostream &operator<<(std::ostream &os, const format &f) { return os << f.str(); }
}
#endif
