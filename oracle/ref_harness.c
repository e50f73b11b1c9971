/*
 * Oracle test infrastructure (not product code).
 *
 * Replay harness linked against the HSMC reference's own object files, which
 * oracle/Makefile compiles unmodified from the reference sources (every file
 * but exec.c, whose main() this harness replaces).  It exposes plain C entry
 * points for ctypes so the tests can run the reference's own code on chosen
 * configurations and chosen proposals:
 *   - set-up exactly as hs_nvt / hs_npt do it (src/nvt.c:32-55, src/npt.c:27-57)
 *   - sweeps through sweep_nvt / sweep_npt (src/nvt.c:201-209, src/npt.c:177-196)
 *   - replayed trial moves through part_move (src/moves.c:27-80) with the
 *     GSL stand-in in script mode, so the reference draws the given values
 *   - the observables' fill routines (src/compute_rdf.c:110-128,
 *     src/compute_press.c:123-165 and :243-273, src/compute_widom_chem_pot.c:44-71,
 *     src/compute_order_parameter.c:82-127)
 * The file-scope statics read below are made linkable by the Makefile with
 * objcopy --globalize-symbol on the compiled objects; the sources are not
 * touched.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "read_input.h"
#include "sim_info.h"
#include "rng.h"
#include "cell_list.h"
#include "moves.h"
#include "nvt.h"
#include "npt.h"
#include "compute_rdf.h"
#include "compute_press.h"
#include "compute_widom_chem_pot.h"
#include "compute_order_parameter.h"
#include "cluster_nvt.h"
#include "cavity_nvt.h"
#include "gsl/gsl_rng.h"

/* Globalised statics of the reference objects. */
extern unsigned long part_moves, vol_moves, acc_part_moves, rej_part_moves, acc_vol_moves, rej_vol_moves;
extern int rdf_hist_nn;
extern double *rdf_hist;
extern int pressv_hist_nn;
extern double *pressv_hist;
extern double pressv_rmax;
extern int presst_hist_nn;
extern double *presst_hist;
extern int wtest;
extern double ql_ave;
extern double *ql;
extern unsigned long r_num_max;
extern int cluster_size;

void global_ql_compute();
void ql_alloc();
void ql_free();

static int ref_ready = 0;
static int rdf_alloc_done = 0, pressv_alloc_done = 0, presst_alloc_done = 0, ql_alloc_done = 0;

/* Read an input file with the reference's parser, then build the box, the
 * lattice, the RNG and the cell list as hs_nvt/hs_npt do. */
int ref_init_from_file(const char *path) {
  if (ref_ready) {
    part_free();
    cell_list_free();
    rng_free();
    ref_ready = 0;
  }
  read_input_file((char *)path);
  sim_box_init(G_IN.type, G_IN.nx, G_IN.ny, G_IN.nz, G_IN.rho);
  part_alloc();
  part_init();
  rng_init();
  cell_list_init(true);
  reset_moves_counters();
  ref_ready = 1;
  return 0;
}

int ref_n(void) { return part_info_get().NN; }

void ref_box(double *out) {
  box_info b = sim_box_info_get();
  cl_info nl = get_cell_list_info();
  out[0] = b.lx;
  out[1] = b.ly;
  out[2] = b.lz;
  out[3] = b.vol;
  out[4] = G_IN.rho;
  out[5] = nl.size_x;
  out[6] = (double)nl.num_x;
  out[7] = G_IN.dr_max;
  out[8] = G_IN.dv_max;
}

void ref_get_config(double *out) {
  config c = part_config_get();
  int n = part_info_get().NN;
  memcpy(out, c, sizeof(double) * 4 * (size_t)n);
}

/* Overwrite positions and rebuild the cell list from scratch. */
void ref_set_config(const double *in) {
  config c = part_config_get();
  int n = part_info_get().NN;
  memcpy(c, in, sizeof(double) * 4 * (size_t)n);
  cell_list_new();
}

void ref_set_steps(double dr_max, double dv_max) {
  G_IN.dr_max = dr_max;
  G_IN.dv_max = dv_max;
}

void ref_sweeps_nvt(int n) {
  for (int i = 0; i < n; i++) sweep_nvt();
}

void ref_sweeps_npt(int n) {
  for (int i = 0; i < n; i++) sweep_npt();
}

void ref_counters(unsigned long *out) {
  out[0] = part_moves;
  out[1] = acc_part_moves;
  out[2] = rej_part_moves;
  out[3] = vol_moves;
  out[4] = acc_vol_moves;
  out[5] = rej_vol_moves;
}

void ref_reset_counters(void) { reset_moves_counters(); }

/* Cavity sampling set up as cavity_hs_nvt does it (src/cavity_nvt.c:27-62):
 * the keyword values, cavity_set_distance, the potential's coefficients
 * (cavity_interaction(0.5, true)), then a fresh cell list. */
void ref_cavity_setup(double pcav, double maxdr, double mindr) {
  G_IN.cavity_pcav = pcav;
  G_IN.cavity_maxdr = maxdr;
  G_IN.cavity_mindr = mindr;
  cavity_set_distance();
  cavity_interaction(0.5, true);
  cell_list_new();
}

void ref_cavity_sweeps(int n) {
  for (int k = 0; k < n; k++) cavity_sweep_nvt();
}

/* cavity_interaction(x, false) for n distances (after ref_cavity_setup). */
void ref_cavity_psi(int n, const double *x, double *out) {
  for (int k = 0; k < n; k++) out[k] = cavity_interaction(x[k], false);
}

/* n calls of cluster_move() (src/cluster_nvt.c:232-310) with the generator;
 * sizes[k] receives the reference's cluster_size after call k. */
void ref_cluster_moves(int n, int *sizes) {
  for (int k = 0; k < n; k++) {
    cluster_move();
    if (sizes) sizes[k] = cluster_size;
  }
}

/* The body of cluster_move after its draws, through the reference's own
 * cluster_move_part, pocket_add and pocket_del, for a given pivot, axis and
 * seed particle; the pocket order comes from the generator.  Returns the
 * cluster size. */
int ref_cluster_move_at(const double *pivot, int axis, int seed_id) {
  double u[3] = {0.0, 0.0, 0.0};
  u[axis] = 1.0;
  int n = part_info_get().NN;
  int *pocket = malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) pocket[i] = -1;
  int count = 0, size = 1;
  cluster_move_part(seed_id, pivot[0], pivot[1], pivot[2], u[0], u[1], u[2]);
  pocket_add(seed_id, pocket, &count);
  while (count > 0) {
    int id = pocket[rng_get_int(count)];
    cluster_move_part(id, pivot[0], pivot[1], pivot[2], u[0], u[1], u[2]);
    pocket_del(id, pocket, &count);
    pocket_add(id, pocket, &count);
    size++;
  }
  free(pocket);
  return size;
}

/* Run part_move() once per entry with scripted draws: ids[k] is returned by
 * rng_get_int and raw[3k..3k+2] by the three rng_get_double calls.
 * accepted[k] receives 1 when the reference accepted the move. */
static unsigned long *widen(const unsigned int *raw, size_t n, int offset_form) {
  unsigned long *w = malloc(sizeof(unsigned long) * (n ? n : 1));
  for (size_t k = 0; k < n; k++) w[k] = offset_form ? 2ul * raw[k] + 1ul : raw[k];
  return w;
}

int ref_replay_moves(int n, const int *ids, const unsigned int *raw, int *accepted) {
  unsigned long *w = widen(raw, 3 * (size_t)n, 0);
  hsmc_shim_script_int(ids, (size_t)n);
  hsmc_shim_script_raw(w, 3 * (size_t)n);
  for (int k = 0; k < n; k++) {
    unsigned long before = acc_part_moves;
    part_move();
    accepted[k] = acc_part_moves != before;
  }
  hsmc_shim_script_off();
  free(w);
  return 0;
}

/* part_move() driven by the device's draws: with the generator maximum set to
 * 2^33 and the draw 2r + 1, rng_get_double returns (2r + 1) / 2^33, so the
 * reference forms u - 0.5 = (2r - 2^32 + 1) * 2^-33 exactly as the device
 * does.  The maximum is restored afterwards. */
int ref_replay_moves_offsets(int n, const int *ids, const unsigned int *raw, int *accepted) {
  unsigned long *w = widen(raw, 3 * (size_t)n, 1);
  unsigned long saved = r_num_max;
  r_num_max = 8589934592ul;
  hsmc_shim_script_int(ids, (size_t)n);
  hsmc_shim_script_raw(w, 3 * (size_t)n);
  for (int k = 0; k < n; k++) {
    unsigned long before = acc_part_moves;
    part_move();
    accepted[k] = acc_part_moves != before;
  }
  hsmc_shim_script_off();
  r_num_max = saved;
  free(w);
  return 0;
}

/* Cavity trials made by the device, through the reference's own
 * cavity_part_move (src/moves.c:254-330): trial k moves cavity which[k]
 * with the uniforms (2r + 1) / 2^33 of raw[3k..3k+2] and, when draws_acc[k]
 * (the trial reached the Metropolis test), the acceptance uniform from
 * uacc[k]; the particle-type draw is scripted to pick a cavity.
 * accepted[k] receives 1 when the reference accepted the move. */
int ref_cavity_replay(int n, const int *which, const unsigned int *raw, const unsigned int *uacc,
                      const int *draws_acc, int *accepted) {
  unsigned long saved = r_num_max;
  r_num_max = 8589934592ul;
  for (int k = 0; k < n; k++) {
    unsigned long w[5];
    size_t nw = 0;
    w[nw++] = 1ul; /* r_type = 2^-33 <= cavity_pcav: a cavity move */
    for (int d = 0; d < 3; d++) w[nw++] = 2ul * raw[3 * k + d] + 1ul;
    if (draws_acc[k]) w[nw++] = 2ul * uacc[k] + 1ul;
    hsmc_shim_script_int(which + k, 1);
    hsmc_shim_script_raw(w, nw);
    unsigned long before = acc_part_moves;
    cavity_part_move();
    accepted[k] = acc_part_moves != before;
    if (hsmc_shim_script_left_raw() != 0) {
      hsmc_shim_script_off();
      r_num_max = saved;
      return -1; /* the reference consumed fewer draws than scripted */
    }
  }
  hsmc_shim_script_off();
  r_num_max = saved;
  return 0;
}

/* The reference's overlap test for particle i placed at (x,y,z), with the cell
 * list left as it is (the state part_move tests in, src/moves.c:51-60). */
int ref_check_overlap_at(int i, double x, double y, double z) {
  config c = part_config_get();
  double ox = c[i][1], oy = c[i][2], oz = c[i][3];
  c[i][1] = x;
  c[i][2] = y;
  c[i][3] = z;
  int ov = check_overlap(i, 1.0, 1.0, 1.0) ? 1 : 0;
  c[i][1] = ox;
  c[i][2] = oy;
  c[i][3] = oz;
  return ov;
}

/* Full scaled overlap scan as vol_move and presst_compute_hist run it. */
int ref_scan_overlap(double sf) {
  int n = part_info_get().NN;
  for (int i = 0; i < n; i++)
    if (check_overlap(i, sf, sf, sf)) return 1;
  return 0;
}

/* One vol_move() with scripted uniforms (raw[0] for the volume, raw[1] for the
 * acceptance test when it is drawn).  Returns 1 when accepted. */
int ref_vol_move_replay(const unsigned int *raw, int n_raw) {
  unsigned long *w = widen(raw, (size_t)n_raw, 0);
  hsmc_shim_script_raw(w, (size_t)n_raw);
  unsigned long before = acc_vol_moves;
  vol_move();
  hsmc_shim_script_off();
  free(w);
  return acc_vol_moves != before;
}

/* g(r) pair counts (the histogram before normalisation) with the cutoff
 * limited to half the box as compute_rdf does on its first call. */
int ref_rdf_counts(double dr, double rmax, double *out, int max_bins, double *rmax_used) {
  box_info b = sim_box_info_get();
  G_IN.rdf_dr = dr;
  G_IN.rdf_rmax = rmax;
  double side = b.lx;
  if (side < b.ly) side = b.ly;
  if (side < b.lz) side = b.lz;
  if (side < 2.0 * G_IN.rdf_rmax) G_IN.rdf_rmax = side / 2.0;
  if (rdf_alloc_done) rdf_hist_free();
  rdf_hist_alloc();
  rdf_alloc_done = 1;
  rdf_hist_init();
  if (rdf_hist_nn > max_bins) return -1;
  rdf_hist_compute();
  memcpy(out, rdf_hist, sizeof(double) * (size_t)rdf_hist_nn);
  if (rmax_used) *rmax_used = G_IN.rdf_rmax;
  return rdf_hist_nn;
}

/* Virial-route contact histogram (before normalisation). */
int ref_pressv_counts(double dr, double *out, int max_bins, double *rmax_used) {
  G_IN.pressv_dr = dr;
  if (pressv_alloc_done) pressv_hist_free();
  pressv_hist_alloc();
  pressv_alloc_done = 1;
  pressv_hist_init();
  if (pressv_hist_nn > max_bins) return -1;
  pressv_compute_hist();
  memcpy(out, pressv_hist, sizeof(double) * (size_t)pressv_hist_nn);
  if (rmax_used) *rmax_used = pressv_rmax;
  return pressv_hist_nn;
}

/* Thermodynamic-route non-overlap indicators, one per compression step. */
int ref_presst_counts(double dxi, double xi_max, double *out, int max_n) {
  G_IN.presst_dxi = dxi;
  G_IN.presst_xi_max = xi_max;
  if (presst_alloc_done) presst_hist_free();
  presst_hist_alloc();
  presst_alloc_done = 1;
  presst_hist_init();
  if (presst_hist_nn > max_n) return -1;
  presst_compute_hist();
  memcpy(out, presst_hist, sizeof(double) * (size_t)presst_hist_nn);
  return presst_hist_nn;
}

/* Widom insertions with scripted uniforms (3 per insertion); returns the
 * number of insertions without overlap. */
int ref_widom(int n, const unsigned int *raw) {
  unsigned long *w = widen(raw, 3 * (size_t)n, 0);
  G_IN.mu_insertions = n;
  hsmc_shim_script_raw(w, 3 * (size_t)n);
  widom_insertion();
  hsmc_shim_script_off();
  free(w);
  return wtest;
}

/* Widom insertions drawing from the generator itself. */
int ref_widom_rng(int n) {
  G_IN.mu_insertions = n;
  widom_insertion();
  return wtest;
}

/* Steinhardt q_l per particle and its mean, with the cutoff clipped to the
 * cell size as compute_op does on its first call. */
double ref_ql(int l, double rc, double *per_particle, double *rc_used) {
  cl_info nl = get_cell_list_info();
  G_IN.ql_order = l;
  G_IN.ql_rmax = rc;
  double side = nl.size_x;
  if (side < nl.size_y) side = nl.size_y;
  if (side < nl.size_z) side = nl.size_z;
  if (side < G_IN.ql_rmax) G_IN.ql_rmax = side;
  if (ql_alloc_done) ql_free();
  ql_alloc();
  ql_alloc_done = 1;
  global_ql_compute();
  if (per_particle) memcpy(per_particle, ql, sizeof(double) * (size_t)part_info_get().NN);
  if (rc_used) *rc_used = G_IN.ql_rmax;
  return ql_ave;
}

/* Raw generator output, for known-answer checks of the stand-in. */
void ref_rng_raw(unsigned long seed, int n, unsigned int *out) {
  gsl_rng *r = gsl_rng_alloc(gsl_rng_mt19937);
  gsl_rng_set(r, seed);
  for (int i = 0; i < n; i++) out[i] = (unsigned int)gsl_rng_get(r);
  gsl_rng_free(r);
}

int ref_rng_uniform_int(unsigned long seed, unsigned long range, int n, int *out) {
  gsl_rng *r = gsl_rng_alloc(gsl_rng_mt19937);
  gsl_rng_set(r, seed);
  for (int i = 0; i < n; i++) out[i] = (int)gsl_rng_uniform_int(r, range);
  gsl_rng_free(r);
  return 0;
}
