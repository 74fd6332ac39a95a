// Line searches on the bi-quadratic energy model P(s, t) = sum_{i,j<=2} q[3i+j] s^i t^j along a
// direction pair (stepSize / newtonUpdate, SystemEnergy.h:256-303).  Host code, double only.
//
// Real roots follow the conventions of the reference's Polynomial::Roots
// (Misha/Polynomial.inl:653-708): a constant coefficient below eps = 1e-14 in magnitude is the
// root 0 and the rest is deflated by s; a zero leading coefficient lowers the degree.  Cubics are
// solved in closed form (Numerical Recipes 3rd ed. section 5.6): with a, b, c the monic
// coefficients, Q = (a^2 - 3b)/9 and R = (2a^3 - 9ab + 27c)/54, three real roots (Viete's
// trigonometric form) when R^2 <= Q^3 + eps, else the single real root of Cardano's formula, or a
// double root when the imaginary part of the complex pair is below eps.
#pragma once
#include <algorithm>
#include <cmath>

namespace epr {
namespace poly {

constexpr double kRootEps = 1e-14;

inline int real_roots(const double *p, int deg, double *r)
{
    int found = 0;
    // deflate roots at zero
    while (deg > 0 && std::fabs(p[0]) < kRootEps)
    {
        r[found++] = 0.0;
        p++;
        deg--;
    }
    while (deg > 0 && p[deg] == 0.0) deg--;
    if (deg == 0) return found;
    if (deg == 1)
    {
        r[found++] = -p[0] / p[1];
        return found;
    }
    if (deg == 2)
    {
        const double disc = p[1] * p[1] - 4.0 * p[0] * p[2];
        if (disc < 0) return found;
        if (disc == 0)
        {
            r[found++] = -p[1] / (2.0 * p[2]);
            return found;
        }
        const double sq = std::sqrt(disc);
        r[found++] = (-p[1] - sq) / (2.0 * p[2]);
        r[found++] = (-p[1] + sq) / (2.0 * p[2]);
        return found;
    }
    const double a = p[2] / p[3], b = p[1] / p[3], c = p[0] / p[3];
    const double Q = (a * a - 3.0 * b) / 9.0;
    const double R = (a * (2.0 * a * a - 9.0 * b) + 27.0 * c) / 54.0;
    const double Q3 = Q * Q * Q, R2 = R * R;
    if (R2 <= Q3 + kRootEps)
    {
        const double theta = std::acos(std::min(1.0, std::max(-1.0, R / std::sqrt(Q3))));
        const double m = -2.0 * std::sqrt(Q), third = a / 3.0, tau = 6.283185307179586476925286766559;
        r[found++] = m * std::cos(theta / 3.0) - third;
        r[found++] = m * std::cos((theta + tau) / 3.0) - third;
        r[found++] = m * std::cos((theta - tau) / 3.0) - third;
        return found;
    }
    double A = -std::cbrt(std::fabs(R) + std::sqrt(R2 - Q3));
    if (R < 0) A = -A;
    const double B = (A == 0.0) ? 0.0 : Q / A;
    r[found++] = (A + B) - a / 3.0;
    if (std::fabs(0.5 * std::sqrt(3.0) * (A - B)) < kRootEps) r[found++] = -0.5 * (A + B) - a / 3.0;
    return found;
}

// p[0..4]: coefficients of u -> P(c0 + u d0, c1 + u d1)
inline void restrict_to_line(const double *q, double c0, double d0, double c1, double d1, double *p)
{
    const double s[3][3] = {{1, 0, 0}, {c0, d0, 0}, {c0 * c0, 2 * c0 * d0, d0 * d0}};
    const double t[3][3] = {{1, 0, 0}, {c1, d1, 0}, {c1 * c1, 2 * c1 * d1, d1 * d1}};
    for (int k = 0; k < 5; k++) p[k] = 0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
        {
            const double qij = q[3 * i + j];
            if (qij == 0) continue;
            for (int a = 0; a <= i; a++)
                for (int b = 0; b <= j; b++) p[a + b] += qij * s[i][a] * t[j][b];
        }
}

inline double eval(const double *p, int deg, double u)
{
    double v = p[deg];
    for (int k = deg - 1; k >= 0; k--) v = v * u + p[k];
    return v;
}

// the critical point of the quartic p with the lowest value (the first root on ties)
inline double quartic_min(const double *p)
{
    const double dp[4] = {p[1], 2 * p[2], 3 * p[3], 4 * p[4]};
    double r[3];
    const int n = real_roots(dp, 3, r);
    if (n == 0) return 0.0;
    double best = r[0];
    for (int k = 1; k < n; k++)
        if (eval(p, 4, r[k]) < eval(p, 4, best)) best = r[k];
    return best;
}

// stepSize: argmin_u P(u, u)
inline double step_size(const double *q)
{
    double p[5];
    restrict_to_line(q, 0, 1, 0, 1, p);
    return quartic_min(p);
}

// newtonUpdate: from (0, 0), Newton directions of P each followed by an exact line search;
// stops when the direction's squared length drops below 1e-20
inline void newton_update(const double *q, int steps, double *st)
{
    double c0 = 0, c1 = 0;
    for (int k = 0; k < steps; k++)
    {
        // gradient and Hessian at (c0, c1)
        const double ps[3] = {1, c0, c0 * c0}, pt[3] = {1, c1, c1 * c1};
        const double dps[3] = {0, 1, 2 * c0}, dpt[3] = {0, 1, 2 * c1};
        const double ddps[3] = {0, 0, 2}, ddpt[3] = {0, 0, 2};
        double g0 = 0, g1 = 0, h00 = 0, h01 = 0, h11 = 0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
            {
                const double v = q[3 * i + j];
                g0 += v * dps[i] * pt[j];
                g1 += v * ps[i] * dpt[j];
                h00 += v * ddps[i] * pt[j];
                h11 += v * ps[i] * ddpt[j];
                h01 += v * dps[i] * dpt[j];
            }
        const double det = h00 * h11 - h01 * h01;
        const double d0 = -(h11 * g0 - h01 * g1) / det;
        const double d1 = -(h00 * g1 - h01 * g0) / det;
        if (d0 * d0 + d1 * d1 < 1e-20) break;
        double p[5];
        restrict_to_line(q, c0, d0, c1, d1, p);
        const double u = quartic_min(p);
        c0 += u * d0;
        c1 += u * d1;
    }
    st[0] = c0;
    st[1] = c1;
}

}  // namespace poly
}  // namespace epr
