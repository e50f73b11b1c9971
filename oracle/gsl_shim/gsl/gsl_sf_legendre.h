/*
 * Oracle test infrastructure (not product code).
 *
 * Stand-in for the one GSL special function the HSMC reference calls,
 * gsl_sf_legendre_sphPlm (src/compute_order_parameter.c:202): the associated
 * Legendre function normalised for spherical harmonics,
 *   sqrt((2l+1)/(4 pi) * (l-m)!/(l+m)!) * P_l^m(x),  0 <= m <= l, |x| <= 1,
 * with the Condon-Shortley phase (-1)^m included in P_l^m.
 */
#ifndef HSMC_ORACLE_GSL_SF_LEGENDRE_H
#define HSMC_ORACLE_GSL_SF_LEGENDRE_H

double gsl_sf_legendre_sphPlm(const int l, int m, const double x);

#endif
