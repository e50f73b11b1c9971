/*
 * Observables of the drop-in program: the device fills the histograms and
 * counts; the host normalises and writes them in the reference's formats:
 *   press_virial.dat  (src/compute_press.c:47-82, 170-187, 277-307)
 *   press_thermo.dat, density.dat  (src/compute_press.c:191-273, 311-359)
 *   order_param.dat   (src/compute_order_parameter.c:25-52, 234-252)
 *   chem_pot.dat      (src/compute_widom_chem_pot.c:32-71, 164-182)
 *   rdf_%06d.dat.gz   (src/compute_rdf.c:36-205)
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <zlib.h>

#include "hsmc_host.h"

void host_obs_begin(host_obs_state *s) {
  s->pressv_init = s->presst_init = s->ql_init = s->mu_init = s->rdf_init = true;
}

static double cells_max_side(const host_run *r) {
  double m = r->cells.size_x;
  if (m < r->cells.size_y) m = r->cells.size_y;
  if (m < r->cells.size_z) m = r->cells.size_z;
  return m;
}

/* Shell normalisation of a pair histogram (src/compute_rdf.c:133-150). */
static void normalise(const double *rr, const uint64_t *counts, double *out, int nn, double rho, int n) {
  double dr = rr[1] - rr[0];
  for (int i = 0; i < nn; i++) {
    double r1 = rr[i] - dr / 2.;
    double r2 = rr[i] + dr / 2.;
    double bin_vol = (4. * M_PI / 3.) * (pow(r2, 3.) - pow(r1, 3.));
    out[i] = (double)counts[i] / (bin_vol * rho * n);
  }
}

static FILE *open_or_die(const char *name, bool init, const char *what) {
  FILE *f = fopen(name, init ? "w" : "a");
  if (!f) {
    perror(what);
    exit(EXIT_FAILURE);
  }
  return f;
}

/* ---------------------------------------------------------------- virial */
static int pv_nn;
static double pv_rmax = 1.05;

void host_compute_pressv(host_run *r, host_obs_state *s) {
  if (s->pressv_init) pv_nn = (int)((pv_rmax - 1.0) / r->in.pressv_dr);
  double *rr = malloc(sizeof(double) * (size_t)pv_nn), *g = malloc(sizeof(double) * (size_t)pv_nn);
  uint64_t *cnt = malloc(sizeof(uint64_t) * (size_t)pv_nn);
  if (!rr || !g || !cnt) {
    printf("ERROR: Failed histogram allocation\n");
    exit(EXIT_FAILURE);
  }
  for (int i = 0; i < pv_nn; i++) rr[i] = (i + 1. / 2.) * r->in.pressv_dr + 1.0;
  pv_rmax = r->in.pressv_dr * pv_nn + 1.0;
  if (s->pressv_init && cells_max_side(r) < pv_rmax) {
    printf("ERROR: The size of the cells in the neighbor list does not allow a correct calculation of the pressure, increase to %f\n",
           pv_rmax);
    exit(EXIT_FAILURE);
  }
  host_gpu_check(hsmc_gpu_pressv(r->gpu, r->in.pressv_dr, pv_rmax, pv_nn, cnt), "pressv");
  normalise(rr, cnt, g, pv_nn, r->in.rho, r->pinfo.NN);
  FILE *f = open_or_die("press_virial.dat", s->pressv_init, "Error while creating the file for the virial pressure\n");
  fprintf(f, "######################################\n");
  fprintf(f, "# Bins, volume, number of particles\n");
  fprintf(f, "######################################\n");
  fprintf(f, "%d %.8e %d\n", pv_nn, r->box.vol, r->pinfo.NN);
  fprintf(f, "###############################\n");
  fprintf(f, "# rr, rdf\n");
  fprintf(f, "###############################\n");
  for (int i = 0; i < pv_nn; i++) fprintf(f, "%.8e %.8e\n", rr[i], g[i]);
  fclose(f);
  free(rr);
  free(g);
  free(cnt);
  s->pressv_init = false;
}

/* ---------------------------------------------------------- thermodynamic */
void host_compute_presst(host_run *r, host_obs_state *s) {
  int nn = (int)(r->in.presst_xi_max / r->in.presst_dxi);
  double *xi = malloc(sizeof(double) * (size_t)(nn > 0 ? nn : 1));
  double *sf = malloc(sizeof(double) * (size_t)(nn > 0 ? nn : 1));
  uint64_t *ok = malloc(sizeof(uint64_t) * (size_t)(nn > 0 ? nn : 1));
  if (!xi || !sf || !ok) {
    printf("ERROR: Failed histogram allocation\n");
    exit(EXIT_FAILURE);
  }
  for (int i = 0; i < nn; i++) {
    xi[i] = (i + 1) * r->in.presst_dxi;
    double ratio = 1 - xi[i];
    sf[i] = pow(ratio, 1. / 3.);
  }
  for (int done = 0; done < nn; done += 256) {
    int chunk = nn - done < 256 ? nn - done : 256;
    host_gpu_check(hsmc_gpu_presst(r->gpu, sf + done, chunk, ok + done), "presst");
  }
  FILE *f = open_or_die("press_thermo.dat", s->presst_init, "Error while creating the file for the thermo pressure\n");
  fprintf(f, "######################################\n");
  fprintf(f, "# Bins, volume, number of particles\n");
  fprintf(f, "######################################\n");
  fprintf(f, "%d %.8e %d\n", nn, r->box.vol, r->pinfo.NN);
  fprintf(f, "######################################\n");
  fprintf(f, "# abs(xi), exp(-beta*U)\n");
  fprintf(f, "######################################\n");
  for (int i = 0; i < nn; i++) fprintf(f, "%.8e %.8e\n", xi[i], (double)ok[i]);
  fclose(f);
  if (r->in.press > 0) {
    f = open_or_die("density.dat", s->presst_init, "Error while creating the file for the density\n");
    if (s->presst_init) {
      fprintf(f, "######################################\n");
      fprintf(f, "# Density (each line is one sample)\n");
      fprintf(f, "######################################\n");
    }
    fprintf(f, "%.8e\n", r->in.rho);
    fclose(f);
  }
  free(xi);
  free(sf);
  free(ok);
  s->presst_init = false;
}

/* ------------------------------------------------------ order parameter */
void host_compute_op(host_run *r, host_obs_state *s) {
  if (s->ql_init) {
    double side = cells_max_side(r);
    if (side < r->in.ql_rmax) {
      printf("WARNING: The cutoff for the order parameter was reduced to %f in order to be consistent with the neighbor list size\n",
             side);
      r->in.ql_rmax = side;
    }
  }
  double q = 0.0;
  host_gpu_check(hsmc_gpu_ql(r->gpu, r->in.ql_order, r->in.ql_rmax, &q, NULL), "ql");
  FILE *f = open_or_die("order_param.dat", s->ql_init, "Error while creating the file for the order parameter\n");
  if (s->ql_init) {
    fprintf(f, "###############################################################\n");
    fprintf(f, "# Average order parameter of order %d (each line is one sample)\n", r->in.ql_order);
    fprintf(f, "###############################################################\n");
  }
  fprintf(f, "%.8e\n", q);
  fclose(f);
  s->ql_init = false;
}

/* ------------------------------------------------------------------ Widom */
void host_compute_mu(host_run *r, host_obs_state *s) {
  uint64_t ok = 0;
  host_gpu_check(hsmc_gpu_widom(r->gpu, r->in.mu_insertions, &ok), "widom");
  double mu = ok > 0 ? -log((double)ok / r->in.mu_insertions) : 0.0;
  FILE *f = open_or_die("chem_pot.dat", s->mu_init, "Error while creating the file for the chemical potential\n");
  if (s->mu_init) {
    fprintf(f, "##################################################################################\n");
    fprintf(f, "# Chemical potenital (average over %d insertions, Fraction of accepted insertions)\n",
            r->in.mu_insertions);
    fprintf(f, "##################################################################################\n");
  }
  fprintf(f, "%.8e %.8e\n", mu, (double)ok / r->in.mu_insertions);
  fclose(f);
  s->mu_init = false;
}

/* ------------------------------------------------------------------- g(r) */
static int rdf_nn, rdf_samples, rdf_file_id;

void host_compute_rdf(host_run *r, host_obs_state *s, int sweep) {
  if (s->rdf_init) {
    double side = r->box.lx;
    if (side < r->box.ly) side = r->box.ly;
    if (side < r->box.lz) side = r->box.lz;
    if (side < 2.0 * r->in.rdf_rmax) {
      r->in.rdf_rmax = side / 2.0;
      printf("WARNING: Cutoff for the rdf extraction reduced to %f in order to be consistent with minimum image convention\n",
             r->in.rdf_rmax);
    }
    rdf_nn = (int)((r->in.rdf_rmax - 1.0) / r->in.rdf_dr);
  }
  double *rr = malloc(sizeof(double) * (size_t)rdf_nn), *g = malloc(sizeof(double) * (size_t)rdf_nn);
  uint64_t *cnt = malloc(sizeof(uint64_t) * (size_t)rdf_nn);
  if (!rr || !g || !cnt) {
    printf("ERROR: Failed histogram allocation\n");
    exit(EXIT_FAILURE);
  }
  for (int i = 0; i < rdf_nn; i++) rr[i] = (i + 1. / 2.) * r->in.rdf_dr + 1.0;
  r->in.rdf_rmax = r->in.rdf_dr * rdf_nn + 1.0;
  host_gpu_check(hsmc_gpu_rdf(r->gpu, r->in.rdf_dr, r->in.rdf_rmax, rdf_nn, cnt), "rdf");
  normalise(rr, cnt, g, rdf_nn, r->in.rho, r->pinfo.NN);
  if (s->rdf_init &&
      (double)(r->in.sweep_stat + r->in.sweep_eq) / (r->in.rdf_sample_int * r->in.rdf_samples) > 100000)
    printf("ERROR: Too many (> 100000) rdf files will be produced. Consider increasing number of samples per file\n");
  char name[30];
  snprintf(name, sizeof(name), "rdf_%06d.dat.gz", rdf_file_id);
  gzFile f = Z_NULL;
  if (rdf_samples == 0) f = gzopen(name, "w");
  else if (rdf_samples > 0 && rdf_samples < r->in.rdf_samples) f = gzopen(name, "a");
  if (f == Z_NULL) {
    perror("Error while creating rdf file");
    exit(EXIT_FAILURE);
  }
  gzprintf(f, "######################################\n");
  gzprintf(f, "# Sweep, Bins, volume, number of particles\n");
  gzprintf(f, "######################################\n");
  gzprintf(f, "%d %d %.8e %d\n", sweep, rdf_nn, r->box.vol, r->pinfo.NN);
  gzprintf(f, "###############################\n");
  gzprintf(f, "# rr, rdf\n");
  gzprintf(f, "###############################\n");
  for (int i = 0; i < rdf_nn; i++) gzprintf(f, "%.8e %.8e\n", rr[i], g[i]);
  gzclose(f);
  rdf_samples += 1;
  if (rdf_samples == r->in.rdf_samples) {
    rdf_samples = 0;
    rdf_file_id += 1;
  }
  free(rr);
  free(g);
  free(cnt);
  s->rdf_init = false;
}
