/* Coefficients of the cavity umbrella potential (cavity_coeffs.c), shared by
 * the host C code that computes them and the device code that uses them. */
#ifndef HSMC_CAVITY_COEFFS_H
#define HSMC_CAVITY_COEFFS_H

typedef struct {
  double ay[4];                  /* Grundke-Henderson cubic, x < 1 */
  double AA, mu, etaW, dW;       /* Verlet-Weis amplitude, decay, effective packing fraction and diameter */
  double t_re[3], t_im[3];       /* Percus-Yevick roots */
  double a_re[3], a_im[3];       /* Percus-Yevick weights */
} hsmc_cavity_psi_coeffs;

#ifdef __cplusplus
extern "C" {
#endif
void hsmc_cavity_coeffs(double rho, hsmc_cavity_psi_coeffs *c);
/* The cavity distance sqrt(r2) is compared with [mindr, maxdr]
 * (src/moves.c:293-297, 349).  sqrt is correctly rounded, hence monotone, so
 * sqrt(r2) >= c exactly when r2 >= hsmc_cavity_r2_at_least(c), and
 * sqrt(r2) <= c exactly when r2 <= hsmc_cavity_r2_at_most(c). */
double hsmc_cavity_r2_at_least(double c);
double hsmc_cavity_r2_at_most(double c);
#ifdef __cplusplus
}
#endif

#endif
