/*
 * Ensemble drivers of the drop-in program: hs_nvt / run_nvt
 * (src/nvt.c:30-199), hs_npt / run_npt (src/npt.c:25-175), cluster_hs_nvt /
 * cluster_run_nvt (src/cluster_nvt.c:31-218) and the displacement optimiser
 * (src/optimizer.c:23-166), with the sweeps on the device.  Sampling happens before the sweep of the same index, as in the
 * reference; consecutive sweeps with nothing to sample between them go to
 * the device as one call.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "hsmc_host.h"

static double wall_seconds(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static bool every(int ii, int interval) { return interval > 0 && ii % interval == 0; }

/* Anything at sweep ii that needs the device state up to date? */
static bool sampling_due(const host_input *in, int ii, bool prod, bool npt) {
  if (every(ii, in->restart_write)) return true;
  if (npt && every(ii, in->output_int)) return true; /* prints the density */
  if (!prod) return false;
  if (every(ii, in->config_write) || every(ii, in->presst_sample_int) || every(ii, in->ql_sample_int)) return true;
  if (!npt && (every(ii, in->pressv_sample_int) || every(ii, in->mu_sample_int) || every(ii, in->rdf_sample_int)))
    return true;
  return false;
}

static void run_block(host_run *r, bool prod, int offset, bool npt) {
  const host_input *in = &r->in;
  if (in->output_int <= 0) {
    printf("ERROR: the output interval (keyword out) must be positive\n");
    exit(EXIT_FAILURE);
  }
  int n = prod ? in->sweep_stat : in->sweep_eq;
  host_obs_state obs;
  host_obs_begin(&obs);
  int pending = 0;
  for (int ii = offset; ii < n + offset; ii++) {
    if (sampling_due(in, ii, prod, npt)) {
      host_sweeps(r, pending, npt);
      pending = 0;
    }
    if (!npt && ii == offset) printf("Sweep number\n");
    if (npt && ii == 0) printf("Sweep number  Density\n");
    if (ii % in->output_int == 0) {
      if (npt) printf("%d  %.8f\n", ii, r->in.rho);
      else printf("%d\n", ii);
      fflush(stdout);
    }
    if (every(ii, in->restart_write)) host_write_restart(r, ii);
    if (prod) {
      if (every(ii, in->config_write)) host_write_config(r, ii);
      if (!npt && every(ii, in->pressv_sample_int)) host_compute_pressv(r, &obs);
      if (every(ii, in->presst_sample_int)) host_compute_presst(r, &obs);
      if (every(ii, in->ql_sample_int)) host_compute_op(r, &obs);
      if (!npt && every(ii, in->mu_sample_int)) host_compute_mu(r, &obs);
      if (!npt && every(ii, in->rdf_sample_int)) host_compute_rdf(r, &obs, ii);
    }
    pending++;
  }
  host_sweeps(r, pending, npt);
}

/* opt_nvt (src/optimizer.c:23-64): secant search of dr_max; opt_cavity_nvt
 * (src/optimizer.c:172-212) is the same search over cavity sweeps, printed
 * with a space before the newline of its acceptance line.  The sampling loop
 * and the secant steps run on the device in one call (hsmc_gpu_optimize),
 * with the reference's arithmetic. */
static void opt_nvt_as(host_run *r, bool cavity) {
  host_input *in = &r->in;
  printf("---------------------------------------------------\n");
  printf("Maximum displacement optimization started ...\n");
  printf("Sweeps for optimization: %d\n", in->opt_sweeps);
  printf("Number of samples: %d\n", in->opt_samples);
  double out[4];
  host_gpu_check(hsmc_gpu_set_step(r->gpu, in->dr_max, in->dv_max), "set_step");
  host_gpu_check(hsmc_gpu_optimize(r->gpu, in->opt_sweeps, in->opt_samples, in->opt_part_target,
                                   in->opt_vol_target, out),
                 "hsmc_gpu_optimize");
  in->dr_max = out[0];
  printf("Optimal maximum displacement: %.8f\n", in->dr_max);
  printf(cavity ? "Acceptance ratio: %.8f \n" : "Acceptance ratio: %.8f\n", out[1]);
  printf("Maximum displacement optimization completed\n");
}

static void opt_nvt(host_run *r) { opt_nvt_as(r, false); }

/* opt_npt (src/optimizer.c:83-148): secant search of dr_max and dv_max, on
 * the device in one call as above. */
static void opt_npt(host_run *r) {
  host_input *in = &r->in;
  printf("---------------------------------------------------\n");
  printf("Maximum displacement optimization started ...\n");
  printf("Sweeps for optimization: %d\n", in->opt_sweeps);
  printf("Number of samples: %d\n", in->opt_samples);
  double out[4];
  host_gpu_check(hsmc_gpu_set_step(r->gpu, in->dr_max, in->dv_max), "set_step");
  host_gpu_check(hsmc_gpu_optimize(r->gpu, in->opt_sweeps, in->opt_samples, in->opt_part_target,
                                   in->opt_vol_target, out),
                 "hsmc_gpu_optimize");
  in->dr_max = out[0];
  in->dv_max = out[2];
  double b[5];
  host_gpu_check(hsmc_gpu_get_box(r->gpu, b), "get_box");
  r->in.rho = b[4];
  r->box.lx = b[0];
  r->box.ly = b[1];
  r->box.lz = b[2];
  r->box.vol = b[3];
  printf("Optimal maximum particle displacement: %.8f\n", in->dr_max);
  printf("Acceptance ratio: %.8f \n", out[1]);
  printf("Optimal maximum volume deformation: %.8f\n", in->dv_max);
  printf("Acceptance ratio: %.8f \n", out[3]);
  printf("Maximum displacement optimization completed\n");
}

static void print_summary(const host_run *r, double seconds, bool npt) {
  const uint64_t *c = r->counters;
  printf("---------------------------------------------------\n");
  printf("-- Particle moves: %.8e\n", (double)c[HSMC_CNT_MOVES]);
  printf("   Acceptance percentage: %f\n", (double)c[HSMC_CNT_ACCEPTED] / ((double)c[HSMC_CNT_MOVES]));
  printf("   Rejection percentage: %f\n", (double)c[HSMC_CNT_REJECTED] / ((double)c[HSMC_CNT_MOVES]));
  if (npt) {
    printf("-- Volume moves: %.8e\n", (double)c[HSMC_CNT_VOL_MOVES]);
    printf("   Acceptance percentage: %f\n", (double)c[HSMC_CNT_VOL_ACCEPTED] / ((double)c[HSMC_CNT_VOL_MOVES]));
    printf("   Rejection percentage: %f\n", (double)c[HSMC_CNT_VOL_REJECTED] / ((double)c[HSMC_CNT_VOL_MOVES]));
  }
  printf("Elapsed time: %f seconds\n", seconds);
}

static void start_system(host_run *r) {
  if (r->in.restart_read == 0) {
    host_box_init(r, r->in.type, r->in.nx, r->in.ny, r->in.nz, r->in.rho);
    host_part_alloc(r);
    host_part_init(r);
  } else {
    host_read_restart(r, r->in.restart_name);
  }
  host_print_sim_info(r);
  host_cells_init(r, true);
  host_gpu_open(r);
  host_gpu_upload(r);
}

static void simulate(host_run *r, bool npt) {
  double t0 = wall_seconds();
  host_reset_counters(r);
  printf("---------------------------------------------------\n");
  printf("Equilibration...\n");
  run_block(r, false, 0, npt);
  printf("Equilibration completed.\n");
  printf("---------------------------------------------------\n");
  printf("Production...\n");
  run_block(r, true, r->in.sweep_eq, npt);
  printf("Production completed.\n");
  print_summary(r, wall_seconds() - t0, npt);
  hsmc_gpu_destroy(r->gpu);
  r->gpu = NULL;
  free(r->conf);
  r->conf = NULL;
}

void host_nvt(host_run *r) {
  start_system(r);
  if (r->in.opt_flag == 1) {
    opt_nvt(r);
    host_part_init(r);
    host_cells_init(r, false);
    host_gpu_upload(r);
  }
  simulate(r, false);
}

/* n cluster sweeps of cluster_moves_sweep moves each (cluster_sweep_nvt,
 * src/cluster_nvt.c:221-228); *last receives the size of the last cluster. */
static void cluster_sweeps(host_run *r, int n, int *last) {
  long long total = (long long)n * r->in.cluster_moves_sweep;
  const long long chunk = 1 << 16;
  int64_t *sizes = malloc(sizeof(int64_t) * (size_t)(total < chunk ? (total > 0 ? total : 1) : chunk));
  while (total > 0) {
    const int k = (int)(total < chunk ? total : chunk);
    host_gpu_check(hsmc_gpu_cluster_moves(r->gpu, k, sizes, NULL), "cluster moves");
    *last = (int)sizes[k - 1];
    total -= k;
  }
  free(sizes);
}

static void cluster_block(host_run *r, bool prod, int offset, int *last) {
  const host_input *in = &r->in;
  if (in->output_int <= 0) {
    printf("ERROR: the output interval (keyword out) must be positive\n");
    exit(EXIT_FAILURE);
  }
  int n = prod ? in->sweep_stat : in->sweep_eq;
  host_obs_state obs;
  host_obs_begin(&obs);
  int pending = 0;
  for (int ii = offset; ii < n + offset; ii++) {
    if (ii % in->output_int == 0 || sampling_due(in, ii, prod, false)) {
      cluster_sweeps(r, pending, last);
      pending = 0;
    }
    if (ii == offset) printf("Sweep number, cluster size\n ");
    if (ii % in->output_int == 0) {
      printf("%d %d\n", ii, *last);
      fflush(stdout);
    }
    if (every(ii, in->restart_write)) host_write_restart(r, ii);
    if (prod) {
      if (every(ii, in->config_write)) host_write_config(r, ii);
      if (every(ii, in->pressv_sample_int)) host_compute_pressv(r, &obs);
      if (every(ii, in->presst_sample_int)) host_compute_presst(r, &obs);
      if (every(ii, in->ql_sample_int)) host_compute_op(r, &obs);
      if (every(ii, in->mu_sample_int)) host_compute_mu(r, &obs);
      if (every(ii, in->rdf_sample_int)) host_compute_rdf(r, &obs, ii);
    }
    pending++;
  }
  cluster_sweeps(r, pending, last);
}

void host_cluster(host_run *r) {
  start_system(r);
  double t0 = wall_seconds();
  host_reset_counters(r);
  /* local sweeps so that a perfect crystal is not rotated */
  host_sweeps(r, r->in.cluster_init_step, false);
  int last = 0;
  printf("---------------------------------------------------\n");
  printf("Equilibration...\n");
  cluster_block(r, false, 0, &last);
  printf("Equilibration completed.\n");
  printf("---------------------------------------------------\n");
  printf("Production...\n");
  cluster_block(r, true, r->in.sweep_eq, &last);
  printf("Production completed.\n");
  printf("Elapsed time: %f seconds\n", wall_seconds() - t0);
  hsmc_gpu_destroy(r->gpu);
  r->gpu = NULL;
  free(r->conf);
  r->conf = NULL;
}

/* --------------------------------------------------------- cavity sampling */

/* cavity_set_distance (src/cavity_nvt.c:172-186) on the host copy. */
static void cavity_set_distance(host_run *r) {
  double ave = (r->in.cavity_maxdr + r->in.cavity_mindr) / 2.0;
  r->conf[1][1] = r->conf[0][1];
  r->conf[1][2] = r->conf[0][2];
  r->conf[1][3] = r->conf[0][3] + ave;
  if (r->conf[1][3] > r->box.lz) r->conf[1][3] -= r->box.lz;
  else if (r->conf[1][3] < 0.0) r->conf[1][3] += r->box.lz;
}

/* cavity_psi_output (src/cavity_nvt.c:191-212), with psi as the device
 * evaluates it. */
static void cavity_psi_output(host_run *r) {
  FILE *fid = fopen("cavity_psi.dat", "w");
  if (fid == NULL) {
    perror("Error while creating the file for the cavity potential\n");
    exit(EXIT_FAILURE);
  }
  fprintf(fid, "#########################################################\n");
  fprintf(fid, "# Interaction potential  between the cavities \n");
  fprintf(fid, "# Distance, potential\n");
  fprintf(fid, "#########################################################\n");
  int n_points = (int)((r->in.cavity_maxdr - r->in.cavity_mindr) / r->in.cavity_out_dr);
  if (n_points > 0) {
    double *x = malloc(sizeof(double) * (size_t)n_points), *psi = malloc(sizeof(double) * (size_t)n_points);
    double xx = r->in.cavity_mindr;
    for (int ii = 0; ii < n_points; ii++) {
      x[ii] = xx;
      xx += r->in.cavity_out_dr;
    }
    host_gpu_check(hsmc_gpu_cavity_psi(r->gpu, x, n_points, psi), "cavity psi");
    for (int ii = 0; ii < n_points; ii++) fprintf(fid, "%.8e %.8e\n", x[ii], psi[ii]);
    free(x);
    free(psi);
  }
  fclose(fid);
}

/* cavity_dist_output (src/cavity_nvt.c:217-237): compute_dist(0, 1). */
static void cavity_dist_output(host_run *r, bool init) {
  host_gpu_download(r);
  double l[3] = {r->box.lx, r->box.ly, r->box.lz}, s2 = 0.0;
  double d[3];
  for (int k = 0; k < 3; k++) {
    d[k] = r->conf[0][1 + k] - r->conf[1][1 + k];
    if (d[k] > l[k] / 2.0) d[k] -= l[k];
    else if (d[k] < -l[k] / 2.0) d[k] += l[k];
  }
  s2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  FILE *fid = fopen("cavity_distance.dat", init ? "w" : "a");
  if (fid == NULL) {
    perror("Error while creating the file for the cavity distance\n");
    exit(EXIT_FAILURE);
  }
  if (init) {
    fprintf(fid, "#########################################################\n");
    fprintf(fid, "# Distance between the cavities (each line is one sample)\n");
    fprintf(fid, "#########################################################\n");
  }
  fprintf(fid, "%.8e\n", sqrt(s2));
  fclose(fid);
}

/* cavity_run_nvt (src/cavity_nvt.c:101-158) */
static void cavity_block(host_run *r, bool prod, int offset, bool *dist_init) {
  const host_input *in = &r->in;
  if (in->output_int <= 0) {
    printf("ERROR: the output interval (keyword out) must be positive\n");
    exit(EXIT_FAILURE);
  }
  int n = prod ? in->sweep_stat : in->sweep_eq;
  int pending = 0;
  for (int ii = offset; ii < n + offset; ii++) {
    const bool dist = prod && every(ii, in->cavity_sample_int);
    if (every(ii, in->restart_write) || (prod && every(ii, in->config_write)) || dist) {
      host_sweeps(r, pending, false);
      pending = 0;
    }
    if (ii == 0) printf("Sweep number\n");
    if (ii % in->output_int == 0) {
      printf("%d\n", ii);
      fflush(stdout);
    }
    if (every(ii, in->restart_write)) host_write_restart(r, ii);
    if (prod) {
      if (every(ii, in->config_write)) host_write_config(r, ii);
      if (dist) {
        cavity_dist_output(r, *dist_init);
        *dist_init = false;
      }
    }
    pending++;
  }
  host_sweeps(r, pending, false);
}

void host_cavity(host_run *r) {
  if (r->in.restart_read == 0) {
    host_box_init(r, r->in.type, r->in.nx, r->in.ny, r->in.nz, r->in.rho);
    host_part_alloc(r);
    host_part_init(r);
    cavity_set_distance(r);
  } else {
    host_read_restart(r, r->in.restart_name);
  }
  host_print_sim_info(r);
  host_cells_init(r, true);
  host_gpu_open(r);
  host_gpu_upload(r);
  cavity_psi_output(r);
  if (r->in.opt_flag == 1) {
    opt_nvt_as(r, true);
    host_part_init(r);
    cavity_set_distance(r);
    host_cells_init(r, false);
    host_gpu_upload(r);
  }
  double t0 = wall_seconds();
  host_reset_counters(r);
  bool dist_init = true;
  printf("---------------------------------------------------\n");
  printf("Equilibration...\n");
  cavity_block(r, false, 0, &dist_init);
  printf("Equilibration completed.\n");
  printf("---------------------------------------------------\n");
  printf("Production...\n");
  cavity_block(r, true, r->in.sweep_eq, &dist_init);
  printf("Production completed.\n");
  print_summary(r, wall_seconds() - t0, false);
  hsmc_gpu_destroy(r->gpu);
  r->gpu = NULL;
  free(r->conf);
  r->conf = NULL;
}

void host_npt(host_run *r) {
  start_system(r);
  if (r->in.opt_flag == 1) {
    double rho_start = r->in.rho;
    opt_npt(r);
    r->in.rho = rho_start;
    host_box_init(r, r->in.type, r->in.nx, r->in.ny, r->in.nz, rho_start);
    host_part_init(r);
    host_cells_init(r, false);
    /* the box changed back: a fresh device context for the lattice start */
    uint64_t st[4];
    host_gpu_check(hsmc_gpu_rng_state(r->gpu, st), "rng_state");
    memcpy(r->rng_host, st, sizeof(st));
    r->have_rng = true;
    host_gpu_open(r);
    host_gpu_upload(r);
  }
  simulate(r, true);
}
