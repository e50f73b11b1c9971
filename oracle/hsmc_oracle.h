/*
 * Oracle test infrastructure (not product code).
 *
 * CPU restatement of the HSMC reference algorithm for the local-move
 * hard-sphere Monte Carlo path: MT19937 draws with GSL conventions, the FCC
 * start, the fixed-capacity cell list, single-particle moves, NpT volume
 * moves, and the observables' fill loops.  Every function follows the
 * reference file:line cited beside it in hsmc_oracle.c, with the same
 * floating-point operation order, so a run with the same seed reproduces the
 * reference's trajectory bit for bit.  Only the tests, the smoke check and
 * the benchmark's CPU-baseline leg load this library; the GPU product never
 * calls it.
 */
#ifndef HSMC_ORACLE_H
#define HSMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hso_sim hso_sim;

/* Error codes (0 = ok). */
enum {
  HSO_OK = 0,
  HSO_ERR_ALLOC = 1,
  HSO_ERR_CELL_OVERFLOW = 2,
  HSO_ERR_CELL_TOO_SMALL = 3,
  HSO_ERR_INIT_OVERLAP = 4,
  HSO_ERR_CELL_DELETE = 5,
  HSO_ERR_ARG = 6
};

hso_sim *hso_create(double rho, int nx, int ny, int nz, int type, double neigh_dr, int neigh_max_part,
                    double dr_max, double dv_max, double press, unsigned long seed, int *err);
void hso_destroy(hso_sim *s);
int hso_n(const hso_sim *s);
void hso_box(const hso_sim *s, double *out9);
void hso_get_config(const hso_sim *s, double *out);
int hso_set_config(hso_sim *s, const double *in);
int hso_reset_lattice(hso_sim *s);
void hso_set_steps(hso_sim *s, double dr_max, double dv_max);
int hso_last_error(const hso_sim *s);

int hso_sweeps_nvt(hso_sim *s, int n);
int hso_sweeps_npt(hso_sim *s, int n);
void hso_counters(const hso_sim *s, unsigned long long *out6);
void hso_reset_counters(hso_sim *s);

int hso_replay_moves(hso_sim *s, int n, const int *ids, const uint32_t *raw, int *accepted);

/* Cavity sampling (src/cavity_nvt.c, src/moves.c:254-440, src/analytic.c). */
void hso_cavity_psi(double rho, int n, const double *x, double *out);
void hso_cavity_coeffs(double rho, double *out20);
int hso_cavity_setup(hso_sim *s, double pcav, double maxdr, double mindr);
int hso_cavity_sweeps(hso_sim *s, int n);
int hso_cavity_replay(hso_sim *s, int n, const int *which, const uint32_t *raw, const uint32_t *uacc,
                      int *decision);

/* Geometric cluster moves (src/cluster_nvt.c:221-431). */
int hso_cluster_move_at(hso_sim *s, const double *pivot, int axis, int seed_id, int *size);
int hso_cluster_moves(hso_sim *s, int n, int *sizes);
int hso_replay_moves_offsets(hso_sim *s, int n, const int *ids, const uint32_t *raw, int *accepted);
int hso_check_overlap_at(hso_sim *s, int i, double x, double y, double z);
int hso_scan_overlap(hso_sim *s, double sf);
int hso_vol_move_replay(hso_sim *s, const uint32_t *raw, int n_raw);

int hso_rdf_counts(hso_sim *s, double dr, double rmax, double *out, int max_bins, double *rmax_used);
int hso_pressv_counts(hso_sim *s, double dr, double *out, int max_bins, double *rmax_used);
int hso_presst_counts(hso_sim *s, double dxi, double xi_max, double *out, int max_n);
int hso_presst_counts_sf(hso_sim *s, const double *sf, int n, double *out);
int hso_widom(hso_sim *s, int n, const uint32_t *raw);
int hso_widom_decisions(hso_sim *s, int n, const uint32_t *raw, uint8_t *overlap);
int hso_widom_rng(hso_sim *s, int n);
int hso_widom_points(hso_sim *s, int n, const double *pts, uint8_t *overlap);
double hso_ql(hso_sim *s, int l, double rc, double *per_particle, double *rc_used);
int hso_opt_nvt(hso_sim *s, int opt_sweeps, int opt_samples, double target, double *dr_out, double *acc_out);

void hso_rng_raw(unsigned long seed, int n, uint32_t *out);
void hso_rng_uniform_int(unsigned long seed, unsigned long range, int n, int *out);

/* Grid-free checks used against the GPU (reference distance arithmetic). */
int hso_brute_overlap(const double *conf, int n, double lx, double ly, double lz, int skip, double x, double y,
                      double z);
int hso_brute_pair_hist(const double *conf, int n, double lx, double ly, double lz, double dr, double rmax,
                        int nbins, unsigned long long *counts);

/* Replay of trial moves made by a checkerboard sweep.  Move k moves particle
 * ids[k] by (2r - 2^32 + 1) * 2^-33 * dr_max per axis for the draws
 * r = raw[3k..3k+2] (the reference's part_move arithmetic with u - 0.5 given
 * exactly); the move must stay in the
 * cell cells[k] of the shifted grid described by shift32[3k..3k+2] and the
 * per-axis (nc, length_f32, inv_width_f32).  decision[k] receives
 * 0 = accepted, 1 = rejected for overlap, 2 = rejected for leaving the cell,
 * 3 = the particle was not in cells[k] before the move. */
int hso_replay_checkerboard(hso_sim *s, int n, const int *ids, const uint32_t *raw, const uint32_t *cells,
                            const float *shift32, const int *nc, const float *len32, const float *inv_w32,
                            int *decision);
uint32_t hso_cell_of32(float x32, float shift32, float len32, float inv_w32, int nc);

#ifdef __cplusplus
}
#endif

#endif
