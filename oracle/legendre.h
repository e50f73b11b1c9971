/*
 * Oracle test infrastructure (not product code).
 *
 * Associated Legendre function normalised for spherical harmonics,
 *   Pbar_l^m(x) = sqrt((2l+1)/(4 pi) * (l-m)!/(l+m)!) * P_l^m(x),
 * Condon-Shortley phase included, by the standard recurrences:
 *   Pbar_0^0 = 1/sqrt(4 pi)
 *   Pbar_m^m = -sqrt((2m+1)/(2m)) sqrt(1-x^2) Pbar_{m-1}^{m-1}
 *   Pbar_{m+1}^m = x sqrt(2m+3) Pbar_m^m
 *   Pbar_l^m = a_lm (x Pbar_{l-1}^m - b_lm Pbar_{l-2}^m),
 *     a_lm = sqrt((4l^2-1)/(l^2-m^2)), b_lm = sqrt(((l-1)^2-m^2)/(4(l-1)^2-1)).
 * This is the quantity the reference obtains from gsl_sf_legendre_sphPlm
 * (src/compute_order_parameter.c:202).  Shared by the GSL stand-in and the
 * restatement so both produce identical bits.
 */
#ifndef HSMC_ORACLE_LEGENDRE_H
#define HSMC_ORACLE_LEGENDRE_H

#include <math.h>

static inline double hso_sph_plm(int l, int m, double x) {
  const double s = sqrt((1.0 - x) * (1.0 + x));
  double pmm = 1.0 / sqrt(4.0 * M_PI);
  for (int k = 1; k <= m; k++) pmm *= -sqrt((2.0 * k + 1.0) / (2.0 * k)) * s;
  if (l == m) return pmm;
  double pm1 = x * sqrt(2.0 * m + 3.0) * pmm;
  if (l == m + 1) return pm1;
  double p2 = pmm, p1 = pm1, p = 0.0;
  for (int ll = m + 2; ll <= l; ll++) {
    double a = sqrt((4.0 * ll * ll - 1.0) / ((double)ll * ll - (double)m * m));
    double b = sqrt(((ll - 1.0) * (ll - 1.0) - (double)m * m) / (4.0 * (ll - 1.0) * (ll - 1.0) - 1.0));
    p = a * (x * p1 - b * p2);
    p2 = p1;
    p1 = p;
  }
  return p;
}

#endif
