// roots.hpp -- from-scratch stand-in for the Boost.Math root-finding names the
// reference's BlackScholes.cpp files use (eps_tolerance, bracket_and_solve_root,
// newton_raphson_iterate) plus boost::uintmax_t.  TEST INFRASTRUCTURE for the
// oracle's reference build only.
//
// Follows Boost's documented contract: bracket_and_solve_root(f, guess, factor,
// rising, tol, max_iter) walks guess*factor^k (or guess/factor^k) until f
// changes sign, then narrows the bracket until tol(a, b) holds or max_iter
// evaluations are spent, and returns the final bracket (a, b).  Boost narrows
// with TOMS 748; this stand-in bisects, so the returned midpoint agrees with
// Boost's only to the requested tolerance (2^(1-bits) relative).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <tuple>
#include <utility>

namespace boost {
typedef std::uintmax_t uintmax_t;
namespace math {
namespace tools {

template <class T>
class eps_tolerance {
public:
    eps_tolerance() : eps_(4 * std::numeric_limits<T>::epsilon()) {}
    explicit eps_tolerance(unsigned bits)
    {
        eps_ = (std::max)(T(std::ldexp(1.0, 1 - static_cast<int>(bits))),
                          T(4 * std::numeric_limits<T>::epsilon()));
    }
    bool operator()(const T& a, const T& b) const
    {
        return std::fabs(a - b) <= eps_ * (std::min)(std::fabs(a), std::fabs(b));
    }

private:
    T eps_;
};

template <class F, class T, class Tol>
std::pair<T, T> bracket_and_solve_root(F f, const T& guess, T factor, bool rising, Tol tol,
                                       boost::uintmax_t& max_iter)
{
    boost::uintmax_t count = max_iter;
    T a = guess, b = guess;
    T fa = f(a), fb = fa;
    if (fa == 0) { max_iter = 1; return std::make_pair(a, a); }
    // root lies towards larger x when f is below zero and rising, or above zero and falling
    bool go_up = (fa < 0) == rising;
    boost::uintmax_t used = 1;
    while (true) {
        if (used >= count) throw std::runtime_error("bracket_and_solve_root: unable to bracket root");
        if (go_up) { a = b; fa = fb; b = b * factor; fb = f(b); }
        else { b = a; fb = fa; a = a / factor; fa = f(a); }
        ++used;
        if (fa == 0) { max_iter = used; return std::make_pair(a, a); }
        if (fb == 0) { max_iter = used; return std::make_pair(b, b); }
        if ((fa < 0) != (fb < 0)) break;
    }
    while (!tol(a, b) && used < count) {
        T m = a + (b - a) / 2;
        T fm = f(m);
        ++used;
        if (fm == 0) { a = b = m; break; }
        if ((fm < 0) == (fa < 0)) { a = m; fa = fm; } else { b = m; fb = fm; }
    }
    max_iter = used;
    return std::make_pair(a, b);
}

// newton_raphson_iterate(f, guess, min, max, digits, max_iter), Boost's
// documented contract: f returns (f(x), f'(x)); Newton steps
// x -= f(x) / f'(x); a step that would leave [min, max] (or a zero
// derivative) is replaced by bisection towards the violated bound; the
// iteration stops once the step is below |x| 2^(1-digits) or after max_iter
// evaluations, and returns x.
template <class F, class T>
T newton_raphson_iterate(F f, T guess, T min, T max, int digits, boost::uintmax_t& max_iter)
{
    const T factor = static_cast<T>(std::ldexp(1.0, 1 - digits));
    T x = guess, delta = (std::numeric_limits<T>::max)();
    boost::uintmax_t count = max_iter, used = 0;
    while (used < count) {
        const auto r = f(x);
        ++used;
        const T f0 = std::get<0>(r), f1 = std::get<1>(r);
        if (f0 == 0) break;
        T next;
        if (f1 == 0) {
            next = (f0 > 0) == (delta > 0) ? (x + min) / 2 : (x + max) / 2;
        } else {
            next = x - f0 / f1;
            if (next < min) next = (x + min) / 2;
            if (next > max) next = (x + max) / 2;
        }
        delta = x - next;
        x = next;
        if (std::fabs(delta) <= std::fabs(x) * factor) break;
    }
    max_iter = used;
    return x;
}

template <class F, class T>
T newton_raphson_iterate(F f, T guess, T min, T max, int digits)
{
    boost::uintmax_t it = (std::numeric_limits<boost::uintmax_t>::max)();
    return newton_raphson_iterate(f, guess, min, max, digits, it);
}

}  // namespace tools
}  // namespace math
}  // namespace boost
