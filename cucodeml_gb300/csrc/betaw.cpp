// The discretised beta distribution of omega among sites under codeml's
// site models M7 (beta) and M8 (beta & omega_s): K equal-probability
// categories, each at its median, omega_j = Q((2j + 1) / (2K); p, q) with Q
// the quantile of Beta(p, q) (DiscreteNSsites codeml.c:2728-2770, QuantileBeta
// in tools.c).  Host code.
//
// The regularised incomplete beta I_x(p, q) is evaluated from its continued
// fraction (DLMF 8.17.22) with the modified Lentz method, on the side of the
// mean where it converges (x < (p + 1) / (p + q + 2), otherwise through
// I_x(p, q) = 1 - I_{1-x}(q, p)); the quantile is Newton's iteration on it,
// kept inside a bisection bracket.
#include <cmath>

#include "gbcodeml.h"

namespace {

// continued fraction of DLMF 8.17.22 at (x, a, b), modified Lentz
double beta_cf(double x, double a, double b) {
    const double tiny = 1e-300, eps = 1e-16;
    double f = 1.0, C = 1.0, D = 0.0;
    for (int n = 1; n <= 1000; n++) {
        const int m = n / 2;
        double d;
        if (n % 2 == 0)
            d = m * (b - m) * x / ((a + 2.0 * m - 1.0) * (a + 2.0 * m));
        else
            d = -(a + m) * (a + b + m) * x / ((a + 2.0 * m) * (a + 2.0 * m + 1.0));
        D = 1.0 + d * D;
        if (std::fabs(D) < tiny) D = tiny;
        C = 1.0 + d / C;
        if (std::fabs(C) < tiny) C = tiny;
        D = 1.0 / D;
        const double delta = C * D;
        f *= delta;
        if (std::fabs(delta - 1.0) < eps) break;
    }
    return f;
}

// I_x(a, b); lnB = ln B(a, b)
double inc_beta(double x, double a, double b, double lnB) {
    if (x <= 0.0) return 0.0;
    if (x >= 1.0) return 1.0;
    if (x < (a + 1.0) / (a + b + 2.0))
        return std::exp(a * std::log(x) + b * std::log1p(-x) - lnB) / (a * beta_cf(x, a, b));
    return 1.0 - std::exp(b * std::log1p(-x) + a * std::log(x) - lnB) / (b * beta_cf(1.0 - x, b, a));
}

// x with I_x(a, b) = prob: Newton's iteration from the leading term of I_x
// near 0 (x^a / (a B)) or near 1, inside a bisection bracket that shrinks
// geometrically while its lower end is still 0 (quantiles of small a reach
// far below any fixed step)
double quantile_beta(double prob, double a, double b) {
    const double lnB = std::lgamma(a) + std::lgamma(b) - std::lgamma(a + b);
    double x = std::exp((std::log(prob) + std::log(a) + lnB) / a);
    if (!(x < 0.5)) {
        const double y = std::exp((std::log1p(-prob) + std::log(b) + lnB) / b);
        x = y < 0.5 ? 1.0 - y : a / (a + b);
    }
    double lo = 0.0, hi = 1.0;
    for (int it = 0; it < 400; it++) {
        const double F = inc_beta(x, a, b, lnB) - prob;
        if (F == 0.0) return x;
        if (F < 0.0) lo = x; else hi = x;
        const double dens = std::exp((a - 1.0) * std::log(x) + (b - 1.0) * std::log1p(-x) - lnB);
        double xn = dens > 0.0 && std::isfinite(dens) ? x - F / dens : -1.0;
        if (!(xn > lo && xn < hi)) xn = lo > 0.0 ? 0.5 * (lo + hi) : 1e-3 * hi;
        if (std::fabs(xn - x) <= 1e-15 * x) return xn;
        x = xn;
    }
    return x;
}

}  // namespace

extern "C" int gb_beta_classes(double p, double q, int K, double *omegas, double *props) {
    if (!omegas || !props || K < 1) return GB_ERR_ARG;
    if (!(p > 0.0) || !(q > 0.0) || !std::isfinite(p) || !std::isfinite(q)) return GB_ERR_PARAM;
    for (int j = 0; j < K; j++) {
        omegas[j] = quantile_beta((2.0 * j + 1.0) / (2.0 * K), p, q);
        props[j] = 1.0 / K;
    }
    return GB_OK;
}
