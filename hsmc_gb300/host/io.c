/*
 * Restart and configuration files of the drop-in program.
 *
 * restart_%0Nd.bin keeps the reference's block order and raw layouts
 * (src/io_config.c:28-130): dr_max, dv_max, the box record, the particle
 * record, the N x 4 configuration; the last block holds this engine's
 * random-stream position (4 x uint64: seed, index of the next sweep, Widom
 * calls, cluster moves)
 * where the reference stores its GSL generator state.  config_%06d.dat.gz is
 * written byte-compatibly from a device download (src/io_config.c:134-191).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <zlib.h>

#include "hsmc_host.h"

static bool restart_check = true, config_check = true;
static int config_samples_done = 0, config_file_id = 0;

void host_write_restart(host_run *r, int sweep) {
  if (restart_check) {
    if ((double)(r->in.sweep_stat + r->in.sweep_eq) / (r->in.restart_write) > 100000)
      printf("ERROR: Too many (> 100000) restart files will be produced. Consider writing less often\n");
    restart_check = false;
  }
  int width = (int)ceil(log10(r->in.sweep_stat + r->in.sweep_eq));
  char tmpl[32], name[64];
  snprintf(tmpl, sizeof(tmpl), "restart_%%0%dd.bin", width);
  snprintf(name, sizeof(name), tmpl, sweep);
  FILE *f = fopen(name, "wb");
  if (!f) {
    perror("Error while creating restart file\n");
    exit(EXIT_FAILURE);
  }
  host_gpu_download(r);
  uint64_t st[4];
  host_gpu_check(hsmc_gpu_rng_state(r->gpu, st), "rng_state");
  fwrite(&r->in.dr_max, sizeof(double), 1, f);
  fwrite(&r->in.dv_max, sizeof(double), 1, f);
  fwrite(&r->box, sizeof(host_box), 1, f);
  fwrite(&r->pinfo, sizeof(host_pinfo), 1, f);
  fwrite(r->conf, sizeof(double), (size_t)r->pinfo.NN * 4, f);
  fwrite(st, sizeof(uint64_t), 4, f);
  fclose(f);
}

void host_read_restart(host_run *r, const char *name) {
  printf("Reading data from restart file %s...\n", name);
  FILE *f = fopen(name, "rb");
  if (!f) {
    perror("Error while reading restart file");
    exit(EXIT_FAILURE);
  }
  size_t ok = 1;
  ok &= fread(&r->in.dr_max, sizeof(double), 1, f) == 1;
  ok &= fread(&r->in.dv_max, sizeof(double), 1, f) == 1;
  ok &= fread(&r->box, sizeof(host_box), 1, f) == 1;
  ok &= fread(&r->pinfo, sizeof(host_pinfo), 1, f) == 1;
  if (!ok || r->pinfo.NN <= 0) {
    printf("ERROR: restart file %s is truncated or damaged\n", name);
    exit(EXIT_FAILURE);
  }
  int n = r->pinfo.NN;
  free(r->conf);
  r->conf = malloc(sizeof(*r->conf) * (size_t)n);
  if (!r->conf) {
    printf("ERROR: Failed particle allocation\n");
    exit(EXIT_FAILURE);
  }
  ok &= fread(r->conf, sizeof(double), (size_t)n * 4, f) == (size_t)n * 4;
  ok &= fread(r->rng_host, sizeof(uint64_t), 4, f) == 4;
  fclose(f);
  if (!ok) {
    printf("ERROR: restart file %s is truncated or damaged\n", name);
    exit(EXIT_FAILURE);
  }
  r->have_rng = true;
  r->in.rho = r->pinfo.NN / r->box.vol;
  printf("The following data was initialized via the restart file:\n"
         "- Maximum displacement (override with optimization)\n"
         "- Maximum volume displacement (only for NpT, override with optimization)\n"
         "- Dimensions of the simulation box\n"
         "- Cell list information\n"
         "- Number of particles\n"
         "- Particle's positions\n"
         "- Density\n"
         "- Status of the random number generator\n");
}

void host_write_config(host_run *r, int sweep) {
  if (config_check) {
    if ((double)(r->in.sweep_stat + r->in.sweep_eq) / (r->in.config_write * r->in.config_samples) > 100000)
      printf("ERROR: Too many (> 100000) configuration files will be produced. Consider increasing number of samples per file\n");
    config_check = false;
  }
  char name[30];
  snprintf(name, sizeof(name), "config_%06d.dat.gz", config_file_id);
  gzFile f = Z_NULL;
  if (config_samples_done == 0) f = gzopen(name, "w");
  else if (config_samples_done > 0 && config_samples_done < r->in.config_samples) f = gzopen(name, "a");
  if (f == Z_NULL) {
    perror("Error while creating configuration file");
    exit(EXIT_FAILURE);
  }
  host_gpu_download(r);
  gzprintf(f, "# Sweep number\n");
  gzprintf(f, "%d\n", sweep);
  gzprintf(f, "# Number of particles\n");
  gzprintf(f, "%d\n", r->pinfo.NN);
  gzprintf(f, "# Simulation box size\n");
  gzprintf(f, "%.8f\n", r->box.lx);
  gzprintf(f, "%.8f\n", r->box.ly);
  gzprintf(f, "%.8f\n", r->box.lz);
  gzprintf(f, "# Configuration\n");
  for (int i = 0; i < r->pinfo.NN; i++)
    gzprintf(f, "%d %.8f %.8f %.8f\n", (int)r->conf[i][0], r->conf[i][1], r->conf[i][2], r->conf[i][3]);
  gzclose(f);
  config_samples_done += 1;
  if (config_samples_done == r->in.config_samples) {
    config_samples_done = 0;
    config_file_id += 1;
  }
}
