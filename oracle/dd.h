/*
 * dd.h -- double-double arithmetic (test infrastructure).
 *
 * A value is hi + lo with |lo| <= ulp(hi)/2, giving ~106 bits of significand.
 * Error-free transforms follow Knuth's TwoSum and the FMA-based TwoProd; the
 * sqrt and division use one Newton correction in double-double (the method of
 * Hida, Li & Bailey's QD library).  Used to run the oracle's force model and
 * IAS15 in extended precision so every double path's error can be stated.
 */
#ifndef ORACLE_DD_H
#define ORACLE_DD_H
#include <cmath>

struct dd {
    double hi, lo;
    dd() : hi(0.0), lo(0.0) {}
    dd(double h) : hi(h), lo(0.0) {}
    dd(double h, double l) : hi(h), lo(l) {}
    explicit operator double() const { return hi + lo; }
};

static inline dd dd_two_sum(double a, double b) {
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    return dd(s, e);
}
static inline dd dd_quick_two_sum(double a, double b) {
    double s = a + b;
    return dd(s, b - (s - a));
}
static inline dd dd_two_prod(double a, double b) {
    double p = a * b;
    return dd(p, std::fma(a, b, -p));
}
static inline dd operator+(const dd& a, const dd& b) {
    dd s = dd_two_sum(a.hi, b.hi);
    dd t = dd_two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = dd_quick_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return dd_quick_two_sum(s.hi, s.lo);
}
static inline dd operator-(const dd& a) { return dd(-a.hi, -a.lo); }
static inline dd operator-(const dd& a, const dd& b) { return a + (-b); }
static inline dd operator*(const dd& a, const dd& b) {
    dd p = dd_two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return dd_quick_two_sum(p.hi, p.lo);
}
static inline dd operator/(const dd& a, const dd& b) {
    double q1 = a.hi / b.hi;
    dd r = a - b * dd(q1);
    double q2 = r.hi / b.hi;
    r = r - b * dd(q2);
    double q3 = r.hi / b.hi;
    dd q = dd_quick_two_sum(q1, q2);
    return q + dd(q3);
}
static inline dd& operator+=(dd& a, const dd& b) { a = a + b; return a; }
static inline dd& operator-=(dd& a, const dd& b) { a = a - b; return a; }
static inline dd& operator*=(dd& a, const dd& b) { a = a * b; return a; }
static inline dd& operator/=(dd& a, const dd& b) { a = a / b; return a; }
static inline bool operator<(const dd& a, const dd& b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
static inline bool operator>(const dd& a, const dd& b) { return b < a; }
static inline bool operator<=(const dd& a, const dd& b) { return !(b < a); }
static inline bool operator>=(const dd& a, const dd& b) { return !(a < b); }
static inline bool operator==(const dd& a, const dd& b) { return a.hi == b.hi && a.lo == b.lo; }
static inline bool operator!=(const dd& a, const dd& b) { return !(a == b); }

static inline dd sqrt(const dd& a) {
    if (a.hi <= 0.0) return dd(std::sqrt(a.hi));
    double x = 1.0 / std::sqrt(a.hi);
    double ax = a.hi * x;
    dd d = a - dd_two_prod(ax, ax);
    return dd_two_sum(ax, d.hi * (x * 0.5));
}
static inline dd fabs(const dd& a) { return a.hi < 0.0 ? -a : a; }
static inline dd floor(const dd& a) {
    double h = std::floor(a.hi);
    if (h == a.hi) return dd_quick_two_sum(h, std::floor(a.lo));
    return dd(h);
}
static inline double to_double(const dd& a) { return a.hi + a.lo; }
static inline double to_double(double a) { return a; }
static inline bool dd_isnormal(const dd& a) { return std::isnormal(a.hi); }
/* pow for the Marsden law: exact integer exponents by repeated products,
 * otherwise exp/log in double on the leading part plus a first-order
 * correction from the trailing part. */
static inline dd pow(const dd& x, double y) {
    if (y == std::floor(y) && std::fabs(y) <= 16.0) {
        dd r(1.0), b = x;
        long n = (long)std::fabs(y);
        while (n) { if (n & 1) r = r * b; b = b * b; n >>= 1; }
        return y < 0 ? dd(1.0) / r : r;
    }
    double p = std::pow(x.hi, y);
    return dd(p) + dd(p * y * (x.lo / x.hi));
}
#endif
