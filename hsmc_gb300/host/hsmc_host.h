/*
 * Drop-in host program for the GB300 engine: the HSMC reference's process
 * interface (flags -i/-e/-o, the keyword input file, the stdout messages and
 * the output files) driving the device through include/hsmc_gpu.h.
 *
 * The input structure keeps the reference's fields and defaults
 * (src/read_input.h:4-71, src/read_input.c:71-115) so files written for the
 * reference run unchanged.
 */
#ifndef HSMC_HOST_H
#define HSMC_HOST_H

#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>

#include "hsmc_gpu.h"

typedef struct {
  double rho;
  int nx, ny, nz, type;
  double neigh_dr;
  int neigh_max_part;
  double dr_max;
  int sweep_eq, sweep_stat;
  int output_int;
  double press, dv_max;
  int opt_flag, opt_samples, opt_sweeps;
  double opt_part_target, opt_vol_target;
  unsigned long int seed;
  double cavity_pcav, cavity_maxdr, cavity_mindr, cavity_out_dr;
  int cavity_sample_int;
  int cluster_flag, cluster_moves_sweep, cluster_init_step;
  int restart_read;
  char restart_name[100];
  int restart_write;
  int config_write, config_samples;
  double pressv_dr, presst_xi_max, presst_dxi;
  int pressv_sample_int, presst_sample_int;
  int ql_order, ql_sample_int;
  double ql_rmax;
  int mu_insertions, mu_sample_int;
  int rdf_sample_int, rdf_samples;
  double rdf_dr, rdf_rmax;
} host_input;

/* Box record written to restart files; field order and types as the
 * reference's box_info (src/sim_info.h:11-18) so restart files share the
 * layout of their first blocks. */
typedef struct {
  double vol;
  double lx, ly, lz;
  double min_size;
  double cell_size;
  int cell_x, cell_y, cell_z;
  int cell_type;
} host_box;

typedef struct {
  int NN;
  int Ncell;
} host_pinfo;

/* Geometry of the reference's own cell list (src/cell_list.c:92-131).  The
 * device uses its own grid; this one only decides the reference's checks and
 * cutoff clips (virial cell size, q_l cutoff, the "27 cells" warning). */
typedef struct {
  int num_x, num_y, num_z;
  double size_x, size_y, size_z;
} host_cells;

typedef struct {
  host_input in;
  host_box box;
  host_pinfo pinfo;
  host_cells cells;
  double (*conf)[4];   /* host copy, downloaded on demand */
  hsmc_ctx *gpu;
  uint64_t counters[6];
  uint64_t rng_host[4]; /* stream position read from a restart file */
  bool have_rng;
} host_run;

/* input.c */
void host_input_defaults(host_input *in);
void host_read_input(host_input *in, const char *filename);
void host_print_example(void);

/* state.c */
void host_box_init(host_run *r, int type, int nx, int ny, int nz, double rho);
void host_part_alloc(host_run *r);
void host_part_init(host_run *r);
void host_cells_init(host_run *r, bool init);
void host_print_sim_info(const host_run *r);
void host_gpu_open(host_run *r);
void host_gpu_upload(host_run *r);
void host_gpu_download(host_run *r);
void host_gpu_check(int status, const char *where);
void host_sweeps(host_run *r, int n, bool npt);
void host_reset_counters(host_run *r);

/* observables.c */
typedef struct {
  bool pressv_init, presst_init, ql_init, mu_init, rdf_init;
} host_obs_state;
void host_obs_begin(host_obs_state *s);
void host_compute_pressv(host_run *r, host_obs_state *s);
void host_compute_presst(host_run *r, host_obs_state *s);
void host_compute_op(host_run *r, host_obs_state *s);
void host_compute_mu(host_run *r, host_obs_state *s);
void host_compute_rdf(host_run *r, host_obs_state *s, int sweep);

/* io.c */
void host_write_restart(host_run *r, int sweep);
void host_read_restart(host_run *r, const char *name);
void host_write_config(host_run *r, int sweep);

/* ensembles.c */
void host_nvt(host_run *r);
void host_npt(host_run *r);
void host_cluster(host_run *r);
void host_cavity(host_run *r);

#endif
