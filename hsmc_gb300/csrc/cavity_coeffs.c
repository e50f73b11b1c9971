/*
 * Coefficients of the cavity umbrella potential psi(x) = ln y_GH(x): the
 * Grundke-Henderson cavity function inside the core, ln of the Verlet-Weis
 * g(r) outside it, which rests on the Percus-Yevick solution at an effective
 * packing fraction (coeff_gh, coeff_vw, coeff_py; src/analytic.c:57-75,
 * 103-140, 174-230).  Computed once per context on the host in C99 complex
 * arithmetic, in the reference's operation order; the device evaluates psi
 * from them (cavity.cu).
 */
#include <complex.h>
#include <math.h>

#include "cavity_coeffs.h"

/* Percus-Yevick: the three roots t_k of the Laplace-space denominator and
 * the residue weights a_k at packing fraction eta. */
static void py_roots(double eta, double complex t[3], double complex a[3]) {
  double complex eta2 = eta * eta;
  double complex ometa = 1.0 - eta, ometa2 = ometa * ometa;
  double complex opeta_2 = 1.0 + eta / 2.0;
  double complex op2eta = 1.0 + 2 * eta;
  double complex ff = 3.0 + 3. * eta - eta2;
  double complex eta2_ff2 = (eta2 / ff) * (eta2 / ff);
  double complex tetaff = cpow(2 * eta * ff, 1. / 3.);
  double complex yp = cpow(sqrt(1. + 2. * eta2_ff2) + 1., 1. / 3.);
  double complex ym = -cpow(sqrt(1. + 2. * eta2_ff2) - 1., 1. / 3.);
  double complex jj = cexp((2. / 3.) * M_PI * I);
  double complex rot[3] = {1.0, jj, jj * jj};
  double complex irot[3] = {1.0, 1. / jj, 1. / (jj * jj)};
  for (int k = 0; k < 3; k++) {
    t[k] = k == 0 ? (-2 * eta + tetaff * (yp + ym)) / ometa
                  : (-2 * eta + tetaff * (yp * rot[k] + ym * irot[k])) / ometa;
    double complex L = opeta_2 * t[k] + op2eta;
    double complex S = 3 * ometa2 * t[k] * t[k] + 12. * eta * ometa * t[k] + 18. * eta2;
    a[k] = t[k] * L / S;
  }
}

/* g_PY(x) for x >= sigma (rdf_py, src/analytic.c:143-170). */
static double py_rdf(const double complex t[3], const double complex a[3], double xx, double sigma) {
  double complex xh = xx / sigma;
  double complex g = a[0] * cexp(t[0] * (xh - 1)) + a[1] * cexp(t[1] * (xh - 1)) + a[2] * cexp(t[2] * (xh - 1));
  return creal(g) / creal(xh);
}

void hsmc_cavity_coeffs(double rho, hsmc_cavity_psi_coeffs *c) {
  const double eta = M_PI * rho / 6.0;
  /* Verlet-Weis: effective diameter and packing fraction, amplitude and decay */
  double eta2 = eta * eta;
  double eta3 = eta2 * eta, eta4 = eta2 * eta2;
  double ometa = 1. - eta, ometa3 = ometa * ometa * ometa;
  double ometa4 = ometa3 * ometa;
  double zz_cs = (1 + eta + eta2 - eta3) / ometa3;
  double mu_cs = ometa4 / (1 + 4. * eta + 4. * eta2 - 4. * eta3 + eta4);
  double dW = pow(1 - eta / 16., 1. / 3.);
  double dW3 = dW * dW * dW, dW4 = dW3 * dW;
  double etaW = eta * dW3;
  double op2etaW2 = (1 + 2 * etaW) * (1 + 2 * etaW);
  double ometaW = 1. - etaW;
  double ometaW3 = ometaW * ometaW * ometaW;
  double ometaW4 = ometaW3 * ometaW;
  double mu_py = ometaW4 / op2etaW2;
  double complex t[3], a[3];
  py_roots(etaW, t, a);
  double AA = (zz_cs - 1.0) / (4.0 * eta) - py_rdf(t, a, 1.0, dW);
  double mu = 12 * AA * eta /
              (mu_cs - mu_py +
               (etaW * (27.0 * etaW * (1 + etaW) - 8.0 * dW * op2etaW2 + dW4 * (8.0 + 5.0 * etaW + 5.0 * etaW * etaW))) /
                   (dW4 * (-ometaW3)));
  /* Grundke-Henderson cubic inside the core, matched to g_VW at contact */
  double g1 = py_rdf(t, a, 1.0, dW) + AA;
  double dg1 = -(9. / 2.) * etaW * (1 + etaW) / ometaW3 - AA * (1 + mu);
  c->ay[0] = (8. * eta - 9. * eta2 + 3. * eta3) / ometa3;
  c->ay[1] = -3. * eta * (2. - eta) / ometa3;
  c->ay[2] = -(dg1 / g1) - 3. * c->ay[0] - 2. * c->ay[1] + 3. * log(g1);
  c->ay[3] = 1. / 3. * ((dg1 / g1) - c->ay[1] - 2. * c->ay[2]);
  c->AA = AA;
  c->mu = mu;
  c->etaW = etaW;
  c->dW = dW;
  for (int k = 0; k < 3; k++) {
    c->t_re[k] = creal(t[k]);
    c->t_im[k] = cimag(t[k]);
    c->a_re[k] = creal(a[k]);
    c->a_im[k] = cimag(a[k]);
  }
}

/* The smallest r2 whose root reaches c, and the largest whose root stays
 * within c: stepped to one double at a time from c * c. */
double hsmc_cavity_r2_at_least(double c) {
  if (!(c > 0.0)) return 0.0; /* every r2 >= 0 has a root >= 0 */
  double x = c * c;
  while (sqrt(x) < c) x = nextafter(x, INFINITY);
  while (x > 0.0 && sqrt(nextafter(x, 0.0)) >= c) x = nextafter(x, 0.0);
  return x;
}

double hsmc_cavity_r2_at_most(double c) {
  if (!(c < INFINITY)) return INFINITY;
  if (c < 0.0) return -1.0; /* no r2 >= 0 qualifies */
  double x = c * c;
  while (sqrt(x) > c) x = nextafter(x, 0.0);
  while (isfinite(x) && sqrt(nextafter(x, INFINITY)) <= c) x = nextafter(x, INFINITY);
  return x;
}
