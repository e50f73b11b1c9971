/*
 * Keyword input file, as the reference reads it (src/read_input.c:62-499):
 * one keyword per line followed by space-separated values, '#' or empty
 * lines ignored, unknown keywords and missing values fatal with the
 * reference's messages.  Defaults are the reference's code defaults.
 */
#define _GNU_SOURCE
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hsmc_host.h"

void host_input_defaults(host_input *in) {
  memset(in, 0, sizeof(*in));
  in->rho = 0.5;
  in->nx = in->ny = in->nz = 3;
  in->type = 1;
  in->neigh_dr = 1.0;
  in->neigh_max_part = 10;
  in->dr_max = 0.05;
  in->sweep_eq = 0;
  in->sweep_stat = 0;
  in->output_int = 0;
  in->cavity_pcav = 0;
  in->cavity_maxdr = 1.2;
  in->cavity_mindr = 0;
  in->cavity_out_dr = 0.01;
  in->cavity_sample_int = 100;
  in->cluster_flag = 0;
  in->cluster_moves_sweep = 1;
  in->cluster_init_step = 10000;
  in->restart_read = 0;
  in->restart_write = 0;
  in->config_write = 0;
  in->config_samples = 128;
  in->pressv_dr = 0.01;
  in->pressv_sample_int = 0;
  in->presst_dxi = 0.0001;
  in->presst_xi_max = 0.002;
  in->presst_sample_int = 0;
  in->press = 0;
  in->dv_max = 0.001;
  in->opt_flag = 1;
  in->opt_sweeps = 1000;
  in->opt_samples = 10;
  in->opt_part_target = 0.5;
  in->opt_vol_target = 0.5;
  in->seed = 0;
  in->ql_order = 6;
  in->ql_rmax = 1.5;
  in->ql_sample_int = 0;
  in->mu_sample_int = 0;
  in->mu_insertions = 100;
  in->rdf_dr = 0.01;
  in->rdf_rmax = 10;
  in->rdf_sample_int = 0;
  in->rdf_samples = 100;
}

static void input_error(int kind, const char *line) {
  if (kind == 1) printf("Missing value to key\n");
  else if (kind == 2) printf("Unknown key\n");
  else if (kind == 3) printf("Name of restart file is too long, maximum 100 characters\n");
  printf("Last read line in the input file:\n%s\n", line);
  exit(EXIT_FAILURE);
}

/* Value slots of one keyword: 'd' = double, 'i' = int, 'u' = unsigned long
 * (read through atoi as the reference does), 's' = restart file name. */
typedef struct {
  const char *key;
  const char *kinds;
  size_t off[5];
} keyword;

#define OFF(f) offsetof(host_input, f)

static const keyword KEYWORDS[] = {
    {"rho", "d", {OFF(rho)}},
    {"cells_x", "i", {OFF(nx)}},
    {"cells_y", "i", {OFF(ny)}},
    {"cells_z", "i", {OFF(nz)}},
    {"type", "i", {OFF(type)}},
    {"neigh_list", "di", {OFF(neigh_dr), OFF(neigh_max_part)}},
    {"dr_max", "d", {OFF(dr_max)}},
    {"sweep_eq", "i", {OFF(sweep_eq)}},
    {"sweep_stat", "i", {OFF(sweep_stat)}},
    {"out", "i", {OFF(output_int)}},
    {"npt", "dd", {OFF(press), OFF(dv_max)}},
    {"opt", "iiidd", {OFF(opt_flag), OFF(opt_sweeps), OFF(opt_samples), OFF(opt_part_target), OFF(opt_vol_target)}},
    {"seed", "u", {OFF(seed)}},
    {"cavity", "dddid",
     {OFF(cavity_pcav), OFF(cavity_maxdr), OFF(cavity_mindr), OFF(cavity_sample_int), OFF(cavity_out_dr)}},
    {"cluster", "iii", {OFF(cluster_flag), OFF(cluster_moves_sweep), OFF(cluster_init_step)}},
    {"restart_read", "is", {OFF(restart_read), OFF(restart_name)}},
    {"restart_write", "i", {OFF(restart_write)}},
    {"config_write", "ii", {OFF(config_write), OFF(config_samples)}},
    {"press_virial", "di", {OFF(pressv_dr), OFF(pressv_sample_int)}},
    {"press_thermo", "ddi", {OFF(presst_dxi), OFF(presst_xi_max), OFF(presst_sample_int)}},
    {"ql", "idi", {OFF(ql_order), OFF(ql_rmax), OFF(ql_sample_int)}},
    {"widom", "ii", {OFF(mu_insertions), OFF(mu_sample_int)}},
    {"rdf", "ddii", {OFF(rdf_dr), OFF(rdf_rmax), OFF(rdf_sample_int), OFF(rdf_samples)}},
};

/* A keyword matches with or without the line's trailing newline. */
static int key_is(const char *tok, const char *key) {
  size_t n = strlen(key);
  return strncmp(tok, key, n) == 0 && (tok[n] == '\0' || (tok[n] == '\n' && tok[n + 1] == '\0'));
}

void host_read_input(host_input *in, const char *filename) {
  host_input_defaults(in);
  printf("Reading input data from %s ...\n", filename);
  FILE *fh = fopen(filename, "r");
  if (!fh) {
    printf("Error! Could not open file %s\n", filename);
    exit(EXIT_FAILURE);
  }
  char *line = NULL;
  size_t cap = 0;
  while (getline(&line, &cap, fh) >= 0) {
    if (line[0] == '#' || line[0] == '\n') continue;
    char *tok = strtok(line, " ");
    const keyword *kw = NULL;
    for (size_t k = 0; tok && k < sizeof(KEYWORDS) / sizeof(KEYWORDS[0]); k++)
      if (key_is(tok, KEYWORDS[k].key)) kw = &KEYWORDS[k];
    if (!kw) input_error(2, line);
    for (int v = 0; kw->kinds[v]; v++) {
      char *val = strtok(NULL, " ");
      if (!val) input_error(1, line);
      char *dst = (char *)in + kw->off[v];
      switch (kw->kinds[v]) {
        case 'd': *(double *)dst = atof(val); break;
        case 'i': *(int *)dst = atoi(val); break;
        case 'u': *(unsigned long *)dst = (unsigned long)atoi(val); break;
        case 's': {
          size_t len = strlen(val);
          if (len && val[len - 1] == '\n') val[len - 1] = '\0';
          if (len < 100) strcpy(dst, val);
          else input_error(3, line);
          break;
        }
      }
    }
  }
  free(line);
  fclose(fh);
  printf("Done\n");
  fflush(stdout);
}

void host_print_example(void) {
  fputs(
      "# This is an input file to compute the pressure via the virial route in the   \n"
      "# canonical (NVT) ensemble. The simulation is performed at density 0.5/sigma^3,\n"
      "# with 1000 particles 1e6 sweeps for equilibration and 1e6 sweeps for statistics\n"
      "# Configuration and restart files are written every 1e5 sweeps, output on screen\n"
      "# is printed every 1e4 sweeps\n\n"
      "# Density\nrho 0.5\n\n"
      "# Simulation box\ncells_x 10\ncells_y 10\ncells_z 10\ntype 1\n\n"
      "# Neighbor list\nneigh_list 1.0 10\n\n"
      "# Maximum particle displacement\ndr_max 0.05\n\n"
      "# Optmizer\nopt 1 1000 10 0.5 0.5\n\n"
      "# Pressure via virial\npress_virial 0.002 10 \n\n"
      "# Seed for random number generator\nseed 124787\n\n"
      "# Write restart data\nrestart_write 100000\n\n"
      "# Write configuration to file\nconfig_write 100000 100\n\n"
      "# Number of sweeps for equilibration\nsweep_eq 1000000\n\n"
      "# Number of sweeps for statistics\nsweep_stat 1000000\n\n"
      "# Output interval\nout 10000\n\n",
      stdout);
}
