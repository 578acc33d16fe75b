/*
 * Kepler radial-velocity model used by the CPU oracle (test infrastructure only).
 *
 * The reference's Cython likelihood calls the external twobody C function
 *   void c_rv_from_elements(double *t, double *rv, int N_t, double P, double K,
 *                           double e, double omega, double phi0, double t0,
 *                           double tol, int maxiter)
 * (declared at thejoker/src/fast_likelihood.pyx:27-30, called at :453-455 with
 * K=1, tol=1e-10, maxiter=128).  twobody (>= 0.9.1, not vendored) is absent, so
 * this header declares a function with that exact signature whose body is
 * written here from the mathematics:
 *   M = 2 pi (t - t0) / P - phi0,   E - e sin E = M,
 *   f = 2 atan2(sqrt(1+e) sin(E/2), sqrt(1-e) cos(E/2)),
 *   rv = K (cos(omega + f) + e cos(omega)).
 * The sign convention is pinned by tests/golden/kepler_known_answer.npz, made
 * from the reference's docs/examples/data.ecsv (a noiseless twobody orbit).
 */
#ifndef JOKER_ORACLE_KEPLER_H
#define JOKER_ORACLE_KEPLER_H
#ifdef __cplusplus
extern "C" {
#endif

/* Eccentric anomaly for mean anomaly M (any real) and 0 <= e < 1, converged to
 * double precision by safeguarded Newton iteration on the bracket [M', M'+e]
 * of the reduced anomaly M' in [0, pi]. */
double oracle_eccentric_anomaly(double M, double e);

/* Unit-amplitude RV column value cos(omega+f) + e cos(omega) at mean anomaly M. */
double oracle_rv_unit(double M, double e, double omega);

void c_rv_from_elements(double *t, double *rv, int N_t, double P, double K,
                        double e, double omega, double phi0, double t0,
                        double tol, int maxiter);

#ifdef __cplusplus
}
#endif
#endif
