// Quad-precision stand-in for boost/multiprecision/cpp_dec_float.hpp.
//
// Test infrastructure only: this header lets the reference's own headers
// compile in a container that has no Boost, so that the reference build under
// oracle/_ref/ can produce golden vectors and validate the C restatement of
// the integrand. It is never linked into the product library.
//
// The reference instantiates number<cpp_dec_float<100>> (100 decimal digits).
// Here every instantiation is backed by IEEE binary128 (__float128, 113-bit
// significand, ~34 decimal digits). On the integrand path the multiprecision
// type only touches the double-double prefactor, the sqrt of the Green-matrix
// scale and parameter parsing, so the FP64 outputs the oracle checks are
// unaffected by the narrower significand.
#pragma once

#include <quadmath.h>

#include <cmath>
#include <cstdlib>
#include <limits>
#include <ostream>
#include <sstream>
#include <string>
#include <type_traits>

namespace boost {
namespace multiprecision {

template <unsigned Digits10>
struct cpp_dec_float {};

template <typename Backend>
class number {
public:
    using quad_t = __float128;

    number() : v_(0) {}
    number(const number&) = default;
    number& operator=(const number&) = default;

    template <typename A, typename std::enable_if<std::is_arithmetic<A>::value, int>::type = 0>
    number(A a) : v_(static_cast<quad_t>(a)) {}

    explicit number(const char* text) : v_(parse(text)) {}
    explicit number(const std::string& text) : v_(parse(text.c_str())) {}

    static number from_quad(quad_t q) {
        number r;
        r.v_ = q;
        return r;
    }
    quad_t quad() const { return v_; }

    template <typename A, typename std::enable_if<std::is_arithmetic<A>::value, int>::type = 0>
    explicit operator A() const {
        return static_cast<A>(v_);
    }

    template <typename A>
    A convert_to() const {
        return static_cast<A>(v_);
    }

    std::string str(std::streamsize digits = 0, std::ios_base::fmtflags = std::ios_base::fmtflags(0)) const {
        char buffer[128];
        const int shown = digits > 0 ? static_cast<int>(digits) : 36;
        quadmath_snprintf(buffer, sizeof(buffer), "%.*Qg", shown, v_);
        return std::string(buffer);
    }

    number operator-() const { return from_quad(-v_); }
    number operator+() const { return *this; }

    number& operator+=(const number& o) { v_ += o.v_; return *this; }
    number& operator-=(const number& o) { v_ -= o.v_; return *this; }
    number& operator*=(const number& o) { v_ *= o.v_; return *this; }
    number& operator/=(const number& o) { v_ /= o.v_; return *this; }

    friend number operator+(const number& a, const number& b) { return from_quad(a.v_ + b.v_); }
    friend number operator-(const number& a, const number& b) { return from_quad(a.v_ - b.v_); }
    friend number operator*(const number& a, const number& b) { return from_quad(a.v_ * b.v_); }
    friend number operator/(const number& a, const number& b) { return from_quad(a.v_ / b.v_); }

#define CDET_SHIM_MIXED(op)                                                                       \
    template <typename A, typename std::enable_if<std::is_arithmetic<A>::value, int>::type = 0> \
    friend number operator op(const number& a, A b) { return a op number(b); }                  \
    template <typename A, typename std::enable_if<std::is_arithmetic<A>::value, int>::type = 0> \
    friend number operator op(A a, const number& b) { return number(a) op b; }
    CDET_SHIM_MIXED(+)
    CDET_SHIM_MIXED(-)
    CDET_SHIM_MIXED(*)
    CDET_SHIM_MIXED(/)
#undef CDET_SHIM_MIXED

#define CDET_SHIM_CMP(op)                                                                         \
    friend bool operator op(const number& a, const number& b) { return a.v_ op b.v_; }           \
    template <typename A, typename std::enable_if<std::is_arithmetic<A>::value, int>::type = 0> \
    friend bool operator op(const number& a, A b) { return a.v_ op static_cast<quad_t>(b); }     \
    template <typename A, typename std::enable_if<std::is_arithmetic<A>::value, int>::type = 0> \
    friend bool operator op(A a, const number& b) { return static_cast<quad_t>(a) op b.v_; }
    CDET_SHIM_CMP(<)
    CDET_SHIM_CMP(>)
    CDET_SHIM_CMP(<=)
    CDET_SHIM_CMP(>=)
    CDET_SHIM_CMP(==)
    CDET_SHIM_CMP(!=)
#undef CDET_SHIM_CMP

    friend std::ostream& operator<<(std::ostream& os, const number& x) {
        const std::streamsize precision = os.precision();
        char buffer[128];
        const bool fixed = (os.flags() & std::ios_base::floatfield) == std::ios_base::fixed;
        quadmath_snprintf(buffer, sizeof(buffer), fixed ? "%.*Qf" : "%.*Qg",
                          static_cast<int>(precision > 0 ? precision : 6), x.v_);
        return os << buffer;
    }

private:
    static quad_t parse(const char* text) {
        char* end = nullptr;
        return strtoflt128(text, &end);
    }

    quad_t v_;
};

#define CDET_SHIM_UNARY(name, qfn)                             \
    template <typename B>                                      \
    inline number<B> name(const number<B>& x) {                \
        return number<B>::from_quad(qfn(x.quad()));            \
    }
CDET_SHIM_UNARY(abs, fabsq)
CDET_SHIM_UNARY(fabs, fabsq)
CDET_SHIM_UNARY(acos, acosq)
CDET_SHIM_UNARY(asin, asinq)
CDET_SHIM_UNARY(atan, atanq)
CDET_SHIM_UNARY(ceil, ceilq)
CDET_SHIM_UNARY(cos, cosq)
CDET_SHIM_UNARY(exp, expq)
CDET_SHIM_UNARY(floor, floorq)
CDET_SHIM_UNARY(log, logq)
CDET_SHIM_UNARY(round, roundq)
CDET_SHIM_UNARY(sin, sinq)
CDET_SHIM_UNARY(sqrt, sqrtq)
CDET_SHIM_UNARY(tan, tanq)
#undef CDET_SHIM_UNARY

template <typename B>
inline number<B> atan2(const number<B>& y, const number<B>& x) {
    return number<B>::from_quad(atan2q(y.quad(), x.quad()));
}
template <typename B>
inline number<B> pow(const number<B>& x, const number<B>& y) {
    return number<B>::from_quad(powq(x.quad(), y.quad()));
}
template <typename B, typename A, typename std::enable_if<std::is_arithmetic<A>::value, int>::type = 0>
inline number<B> pow(const number<B>& x, A y) {
    return number<B>::from_quad(powq(x.quad(), static_cast<__float128>(y)));
}
template <typename B>
inline number<B> ldexp(const number<B>& x, int e) {
    return number<B>::from_quad(ldexpq(x.quad(), e));
}
template <typename B>
inline bool isfinite(const number<B>& x) { return finiteq(x.quad()) != 0; }
template <typename B>
inline bool isinf(const number<B>& x) { return isinfq(x.quad()) != 0; }
template <typename B>
inline bool isnan(const number<B>& x) { return isnanq(x.quad()) != 0; }

}  // namespace multiprecision
}  // namespace boost

namespace std {
template <typename B>
class numeric_limits<boost::multiprecision::number<B>> {
public:
    static constexpr bool is_specialized = true;
    static constexpr int digits = 113;
    static constexpr int digits10 = 33;
    static constexpr int max_digits10 = 36;
    static boost::multiprecision::number<B> epsilon() {
        return boost::multiprecision::number<B>::from_quad(ldexpq(1, -112));
    }
    static boost::multiprecision::number<B> min() {
        return boost::multiprecision::number<B>::from_quad(ldexpq(1, -16382));
    }
    static boost::multiprecision::number<B> max() {
        return boost::multiprecision::number<B>::from_quad(ldexpq(2 - ldexpq(1, -112), 16383));
    }
};
}  // namespace std
