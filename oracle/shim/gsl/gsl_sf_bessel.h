/*
 * Stand-in for the one GSL routine the reference's gridder calls
 * (gsl_sf_bessel_I0, lentils/backend/nufft.c:20). GSL is not installed here, so this header
 * lets the reference's own nufft.c compile unmodified, and the oracle port uses the same
 * function so both CPU paths agree.
 *
 * TEST INFRASTRUCTURE: part of the oracle. Nothing on the product path includes it.
 *
 * Method: the defining power series of the modified Bessel function of the first kind,
 *   I0(x) = sum_{k>=0} (x^2/4)^k / (k!)^2      (Abramowitz & Stegun 9.6.12),
 * evaluated by Horner's rule in q = x^2/4 with a term count chosen from |x| so that the
 * dropped tail is below 1e-18 of the sum. Every term is positive, so Horner's rule is
 * forward-stable and the result is accurate to a few ulp. Arguments beyond 60 fall back to
 * summing terms until they stop contributing.
 */
#ifndef LENTILS_ORACLE_GSL_SF_BESSEL_SHIM_H
#define LENTILS_ORACLE_GSL_SF_BESSEL_SHIM_H

#include <math.h>

static inline double lentils_oracle_bessel_i0(double x)
{
    const double q = 0.25 * x * x;
    const double ax = fabs(x);
    int nterms;
    if (ax <= 2.0) nterms = 12;
    else if (ax <= 8.0) nterms = 24;
    else if (ax <= 20.0) nterms = 42;
    else if (ax <= 40.0) nterms = 70;
    else if (ax <= 60.0) nterms = 96;
    else {
        /* adaptive summation for very large arguments */
        double sum = 1.0, term = 1.0;
        for (int k = 1; k < 100000; ++k) {
            term *= q / ((double)k * (double)k);
            sum += term;
            if (term < 1e-18 * sum) break;
        }
        return sum;
    }
    /* Horner in q with coefficients 1/(k!)^2, built from the top term down:
     *   s_K = 1;  s_{k-1} = 1 + q/k^2 * s_k;  I0 = s_0. */
    double s = 1.0;
    for (int k = nterms; k >= 1; --k)
        s = 1.0 + (q / ((double)k * (double)k)) * s;
    return s;
}

/* The name the reference's nufft.c calls. */
static inline double gsl_sf_bessel_I0(double x) { return lentils_oracle_bessel_i0(x); }

#endif
