// CPU check of the double-float arithmetic (hsmc_gb300/csrc/df64.cuh) that
// the q_l kernel runs its recurrences in: the operations against double
// arithmetic, and q_l per particle from the same recurrences in double and in
// double-float on random bond sets (polar bonds included).  Built by
// tests/test_df64.py without contraction.
#include <cmath>
#include <cstdio>
#include <random>
#include "df64.cuh"
using namespace hsmc;
const int LMAX = 12;
double diag[LMAX+1], first[LMAX+1], A[LMAX+1][LMAX+1], B[LMAX+1][LMAX+1];
F2 diagf[LMAX+1], firstf[LMAX+1], Af[LMAX+1][LMAX+1], Bf[LMAX+1][LMAX+1];
void coef() {
  for (int m = 0; m <= LMAX; m++) {
    diag[m] = m > 0 ? sqrt((2.0*m+1.0)/(2.0*m)) : 0.0; first[m] = sqrt(2.0*m+3.0);
    for (int ll = 0; ll <= LMAX; ll++) {
      double den = (double)ll*ll - (double)m*m; A[ll][m] = den > 0 ? sqrt((4.0*ll*ll-1.0)/den) : 0.0;
      double nb = (ll-1.0)*(ll-1.0) - (double)m*m, db = 4.0*(ll-1.0)*(ll-1.0) - 1.0;
      B[ll][m] = (nb >= 0 && db > 0) ? sqrt(nb/db) : 0.0;
      Af[ll][m] = f2_of(A[ll][m]); Bf[ll][m] = f2_of(B[ll][m]);
    }
    diagf[m] = f2_of(-diag[m]); firstf[m] = f2_of(first[m]);
  }
}
void bond_d(double dx, double dy, double dz, int l, double *re, double *im) {
  double r = sqrt(dx*dx+dy*dy+dz*dz), inv_r = 1.0/r, rho = sqrt(dx*dx+dy*dy), inv_rho = rho > 0 ? 1.0/rho : 0;
  double ct = dz*inv_r, st = rho*inv_r, cp = rho > 0 ? dx*inv_rho : 1.0, sp = rho > 0 ? dy*inv_rho : 0.0;
  double pmm = 0.28209479177387814, cm = 1, sm = 0;
  for (int m = 0; m <= l; m++) {
    if (m > 0) { pmm *= -diag[m]*st; double c2 = cm*cp - sm*sp; sm = sm*cp + cm*sp; cm = c2; }
    double plm = pmm;
    if (l > m) { double p2 = pmm, p1 = ct*first[m]*pmm;
      for (int ll = m+2; ll <= l; ll++) { double pn = A[ll][m]*(ct*p1 - B[ll][m]*p2); p2 = p1; p1 = pn; }
      plm = p1; }
    re[m] += plm*cm; im[m] += plm*sm;
  }
}
void bond_f(double dx, double dy, double dz, int l, F2 *re, F2 *im) {
  double r = sqrt(dx*dx+dy*dy+dz*dz), inv_r = 1.0/r, rho = sqrt(dx*dx+dy*dy), inv_rho = rho > 0 ? 1.0/rho : 0;
  F2 ct = f2_of(dz*inv_r), st = f2_of(rho*inv_r), cp = f2_of(rho > 0 ? dx*inv_rho : 1.0), sp = f2_of(rho > 0 ? dy*inv_rho : 0.0);
  F2 pmm = f2_of(0.28209479177387814), cm = F2{1.f, 0.f}, sm = F2{0.f, 0.f};
  for (int m = 0; m <= l; m++) {
    if (m > 0) { pmm = f2_mul(f2_mul(pmm, diagf[m]), st); F2 c2 = f2_sub(f2_mul(cm, cp), f2_mul(sm, sp)); sm = f2_add(f2_mul(sm, cp), f2_mul(cm, sp)); cm = c2; }
    F2 plm = pmm;
    if (l > m) { F2 p2 = pmm, p1 = f2_mul(f2_mul(ct, firstf[m]), pmm);
      for (int ll = m+2; ll <= l; ll++) { F2 pn = f2_mul(Af[ll][m], f2_sub(f2_mul(ct, p1), f2_mul(Bf[ll][m], p2))); p2 = p1; p1 = pn; }
      plm = p1; }
    re[m] = f2_add(re[m], f2_mul(plm, cm)); im[m] = f2_add(im[m], f2_mul(plm, sm));
  }
}
double qfrom(double *re, double *im, int l, int nb) {
  double s = 0; for (int m = 0; m <= l; m++) { double a = re[m]/nb, b = im[m]/nb; s += (m==0?1.0:2.0)*(a*a+b*b); }
  return sqrt(s*(4.0*M_PI/(2*l+1)));
}
extern "C" {

// max |q_df - q_d| over n particles of 6..15 bonds at 1 <= r <= 1.5
double ql_max_error(int l, long n, unsigned long long seed) {
  coef();
  std::mt19937_64 g(seed);
  std::uniform_real_distribution<double> u(-1, 1), rr(1.0, 1.5);
  double maxerr = 0;
  for (long p = 0; p < n; p++) {
    int nb = 6 + (int)(g() % 10);
    double re[13] = {0}, im[13] = {0};
    F2 ref[13], imf[13];
    for (int m = 0; m < 13; m++) ref[m] = imf[m] = F2{0, 0};
    for (int b = 0; b < nb; b++) {
      double x, y, z, n2;
      do { x = u(g); y = u(g); z = u(g); n2 = x * x + y * y + z * z; } while (n2 > 1 || n2 < 1e-6);
      double s = rr(g) / sqrt(n2);
      x *= s; y *= s; z *= s;
      if (p % 1000 == 0 && b == 0) { x = 0; y = 0; }  // polar bonds
      bond_d(x, y, z, l, re, im);
      bond_f(x, y, z, l, ref, imf);
    }
    double re2[13], im2[13];
    for (int m = 0; m < 13; m++) { re2[m] = f2_value(ref[m]); im2[m] = f2_value(imf[m]); }
    const double e = fabs(qfrom(re, im, l, nb) - qfrom(re2, im2, l, nb));
    if (e > maxerr) maxerr = e;
  }
  return maxerr;
}

// the largest relative error of f2_mul and f2_add against double over n
// random pairs of double-float values
void op_max_errors(long n, unsigned long long seed, double *out) {
  std::mt19937_64 g(seed);
  std::uniform_real_distribution<double> u(-4, 4);
  double em = 0, ea = 0;
  for (long k = 0; k < n; k++) {
    const F2 a = f2_of(u(g)), b = f2_of(u(g));
    const double x = f2_value(a), y = f2_value(b);
    const double m = x * y, s = x + y;
    const double dm = fabs(f2_value(f2_mul(a, b)) - m) / fabs(m);
    if (dm > em) em = dm;
    if (fabs(s) > 1e-3) {
      const double da = fabs(f2_value(f2_add(a, b)) - s) / fabs(s);
      if (da > ea) ea = da;
    }
  }
  out[0] = em;
  out[1] = ea;
}
}
