/*
 * CPU oracle (test infrastructure only): Kepler equation and unit-K radial
 * velocity.  See kepler.h for the convention and where it is pinned.
 */
#include <math.h>
#include "kepler.h"

static const double TWO_PI = 6.283185307179586476925286766559;
static const double PI_D = 3.1415926535897932384626433832795;

double oracle_eccentric_anomaly(double M, double e)
{
    /* reduce M to (-pi, pi]; E(-M) = -E(M) */
    double Mr = fmod(M, TWO_PI);
    if (Mr > PI_D) Mr -= TWO_PI;
    if (Mr <= -PI_D) Mr += TWO_PI;
    double sgn = 1.0;
    if (Mr < 0.0) { sgn = -1.0; Mr = -Mr; }
    if (e == 0.0) return sgn * Mr;

    /* f(E) = E - e sin E - Mr is increasing; its root lies in [Mr, min(pi, Mr + e)] */
    double lo = Mr, hi = Mr + e;
    if (hi > PI_D) hi = PI_D;
    double E = (e < 0.8) ? Mr + e * sin(Mr) : PI_D;
    if (E < lo || E > hi) E = 0.5 * (lo + hi);
    for (int it = 0; it < 200; ++it) {
        double s = sin(E), c = cos(E);
        double f = E - e * s - Mr;
        if (f == 0.0) break;
        if (f > 0.0) hi = E; else lo = E;
        double fp = 1.0 - e * c;
        double En = E - f / fp;
        if (!(En > lo && En < hi)) En = 0.5 * (lo + hi);   /* bisection fallback */
        double dE = En - E;
        E = En;
        if (fabs(dE) <= 1e-15 * (1.0 + fabs(E))) break;
    }
    return sgn * E;
}

double oracle_rv_unit(double M, double e, double omega)
{
    double E = oracle_eccentric_anomaly(M, e);
    double f = 2.0 * atan2(sqrt(1.0 + e) * sin(0.5 * E), sqrt(1.0 - e) * cos(0.5 * E));
    return cos(omega + f) + e * cos(omega);
}

void c_rv_from_elements(double *t, double *rv, int N_t, double P, double K,
                        double e, double omega, double phi0, double t0,
                        double tol, int maxiter)
{
    (void)tol; (void)maxiter;   /* always converged to double precision */
    for (int i = 0; i < N_t; ++i) {
        double M = 2.0 * PI_D * (t[i] - t0) / P - phi0;
        rv[i] = K * oracle_rv_unit(M, e, omega);
    }
}
