// normal.hpp -- from-scratch stand-in for the Boost.Math normal distribution
// names the reference's rBergomi/qmc.h uses (boost::math::normal and
// quantile(normal, p)).  TEST INFRASTRUCTURE for the oracle's reference build
// only.
//
// quantile() inverts Phi(x) = erfc(-x / sqrt 2) / 2 to within a few ulps: a
// starting value from Hastings' rational approximation (Abramowitz & Stegun
// 26.2.23, |error| < 4.5e-4), then three Halley steps on Phi(x) = q worked on
// the lower tail (q = min(p, 1 - p), where erfc carries full relative
// accuracy).  Boost computes the same function by its own rational
// approximations, so the two agree to a few ulps, not bit for bit.  The
// oracle's C restatement (rbgo_inv_normal) runs the same steps.
#pragma once
#include <cmath>
#include <limits>

namespace boost {
namespace math {

class normal {
public:
    explicit normal(double mean = 0.0, double sd = 1.0) : mean_(mean), sd_(sd) {}
    double mean() const { return mean_; }
    double standard_deviation() const { return sd_; }

private:
    double mean_, sd_;
};

inline double quantile(const normal& d, double p)
{
    if (!(p > 0.0)) return p == 0.0 ? -std::numeric_limits<double>::infinity() : std::nan("");
    if (!(p < 1.0)) return p == 1.0 ? std::numeric_limits<double>::infinity() : std::nan("");
    const bool upper = p > 0.5;
    const double q = upper ? 1.0 - p : p;  // exact for p >= 1/2
    const double t = std::sqrt(-2.0 * std::log(q));
    double x = -(t - (2.515517 + t * (0.802853 + t * 0.010328)) / (1.0 + t * (1.432788 + t * (0.189269 + t * 0.001308))));
    for (int i = 0; i < 3; ++i) {
        const double e = 0.5 * std::erfc(-x * 0.70710678118654752440) - q;
        const double u = e * 2.50662827463100050242 * std::exp(0.5 * x * x);  // e / phi(x)
        x = x - u / (1.0 + 0.5 * x * u);
    }
    return d.mean() + d.standard_deviation() * (upper ? -x : x);
}

}  // namespace math
}  // namespace boost
