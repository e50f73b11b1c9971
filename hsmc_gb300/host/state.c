/*
 * Host-side state of one run: the box and lattice start with the
 * reference's arithmetic (src/sim_info.c:32-156), the reference's cell-list
 * geometry for its checks (src/cell_list.c:92-131), and the device context.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hsmc_host.h"

void host_gpu_check(int status, const char *where) {
  if (status == HSMC_OK) return;
  printf("%s\n", hsmc_gpu_strerror(status));
  fprintf(stderr, "hsmc: %s failed with status %d\n", where, status);
  exit(EXIT_FAILURE);
}

void host_box_init(host_run *r, int type, int nx, int ny, int nz, double rho) {
  int per_cell;
  if (type == 1) {
    per_cell = 1;
  } else if (type == 2) {
    per_cell = 4;
  } else {
    printf("Unknown lattice type, default to fcc\n");
    per_cell = 4;
  }
  double cell_vol = per_cell / rho;
  double cell_size = pow(cell_vol, 1. / 3.);
  int min_n = nx;
  if (ny < min_n) min_n = ny;
  if (nz < min_n) min_n = nz;
  r->box.cell_x = nx;
  r->box.cell_y = ny;
  r->box.cell_z = nz;
  r->box.lx = nx * cell_size;
  r->box.ly = ny * cell_size;
  r->box.lz = nz * cell_size;
  r->box.min_size = min_n * cell_size;
  r->box.vol = nx * ny * nz * cell_vol;
  r->box.cell_size = cell_size;
  r->box.cell_type = type;
}

void host_part_alloc(host_run *r) {
  int per_cell = (r->box.cell_type == 1) ? 1 : 4;
  if (r->box.cell_type != 1 && r->box.cell_type != 2) printf("Unknown lattice type, default to fcc\n");
  int n = r->box.cell_x * r->box.cell_y * r->box.cell_z * per_cell;
  free(r->conf);
  r->conf = malloc(sizeof(*r->conf) * (size_t)n);
  if (!r->conf) {
    printf("ERROR: Failed particle allocation\n");
    exit(EXIT_FAILURE);
  }
  r->pinfo.Ncell = per_cell;
  r->pinfo.NN = n;
}

static void lattice_error(void) {
  printf("Overlap in the initial configuration. Possible solutions:\n");
  printf("-- If SC lattice was selected, try to change to FCC\n");
  printf("-- If FCC lattice was selected, the selected value of density is unphysical\n");
  exit(EXIT_FAILURE);
}

static void put(host_run *r, int id, double x, double y, double z) {
  r->conf[id][0] = id;
  r->conf[id][1] = x;
  r->conf[id][2] = y;
  r->conf[id][3] = z;
}

void host_part_init(host_run *r) {
  double a = r->box.cell_size;
  int id = 0;
  if (r->box.cell_type == 1) {
    if (a < 1) lattice_error();
    for (int i = 0; i < r->box.cell_x; i++)
      for (int j = 0; j < r->box.cell_y; j++)
        for (int k = 0; k < r->box.cell_z; k++) put(r, id++, i * a, j * a, k * a);
  } else {
    if (a / sqrt(2.0) < 1) lattice_error();
    for (int i = 0; i < r->box.cell_x; i++)
      for (int j = 0; j < r->box.cell_y; j++)
        for (int k = 0; k < r->box.cell_z; k++) {
          put(r, id, i * a, j * a, k * a);
          put(r, id + 1, (i + 0.5) * a, (j + 0.5) * a, k * a);
          put(r, id + 2, (i + 0.5) * a, j * a, (k + 0.5) * a);
          put(r, id + 3, i * a, (j + 0.5) * a, (k + 0.5) * a);
          id += 4;
        }
  }
}

void host_cells_init(host_run *r, bool init) {
  host_cells *c = &r->cells;
  if (init) {
    c->num_x = (int)floor(r->box.lx / r->in.neigh_dr);
    c->num_y = (int)floor(r->box.ly / r->in.neigh_dr);
    c->num_z = (int)floor(r->box.lz / r->in.neigh_dr);
    if (c->num_x * c->num_y * c->num_z < 27) {
      printf("WARNING: The specified cell size has been reduced in order to accomodate 27 cells in the simulation box\n");
      c->num_x = c->num_y = c->num_z = 3;
    }
  }
  c->size_x = r->box.lx / c->num_x;
  c->size_y = r->box.ly / c->num_y;
  c->size_z = r->box.lz / c->num_z;
  if (c->size_x < 1.0 || c->size_y < 1.0 || c->size_z < 1.0) {
    printf("ERROR: size of cells in cell list is smaller than the size of the particles\n");
    exit(EXIT_FAILURE);
  }
}

void host_print_sim_info(const host_run *r) {
  printf("Simulation box size (x, y, z): %.5f %.5f %.5f\n", r->box.lx, r->box.ly, r->box.lz);
  printf("Number of particles: %d\n", r->pinfo.NN);
  if (r->in.press > 0) printf("Pressure: %.8f\n", r->in.press);
}

void host_gpu_open(host_run *r) {
  if (r->gpu) hsmc_gpu_destroy(r->gpu);
  hsmc_params p;
  memset(&p, 0, sizeof(p));
  p.n_particles = r->pinfo.NN;
  p.lattice_type = r->box.cell_type;
  p.cells[0] = r->box.cell_x;
  p.cells[1] = r->box.cell_y;
  p.cells[2] = r->box.cell_z;
  p.rho = r->in.rho;
  p.box[0] = r->box.lx;
  p.box[1] = r->box.ly;
  p.box[2] = r->box.lz;
  p.dr_max = r->in.dr_max;
  p.dv_max = r->in.dv_max;
  p.pressure = r->in.press;
  p.seed = r->in.seed;
  if (r->in.press <= 0 && r->in.cavity_pcav > 0) {
    p.cavity_pcav = r->in.cavity_pcav;
    p.cavity_maxdr = r->in.cavity_maxdr;
    p.cavity_mindr = r->in.cavity_mindr;
  }
  host_gpu_check(hsmc_gpu_create(&p, &r->gpu), "hsmc_gpu_create");
  if (r->have_rng) host_gpu_check(hsmc_gpu_rng_set_state(r->gpu, r->rng_host), "hsmc_gpu_rng_set_state");
}

void host_gpu_upload(host_run *r) {
  host_gpu_check(hsmc_gpu_upload_config(r->gpu, (const double(*)[4])r->conf, r->pinfo.NN), "upload");
}

void host_gpu_download(host_run *r) {
  host_gpu_check(hsmc_gpu_download_config(r->gpu, r->conf, r->pinfo.NN), "download");
}

void host_reset_counters(host_run *r) { memset(r->counters, 0, sizeof(r->counters)); }

void host_sweeps(host_run *r, int n, bool npt) {
  if (n <= 0) return;
  uint64_t c[6];
  host_gpu_check(hsmc_gpu_set_step(r->gpu, r->in.dr_max, r->in.dv_max), "set_step");
  if (npt) host_gpu_check(hsmc_gpu_npt_sweeps(r->gpu, n, c), "npt sweeps");
  else host_gpu_check(hsmc_gpu_sweeps(r->gpu, n, c), "sweeps");
  for (int k = 0; k < 6; k++) r->counters[k] += c[k];
  if (npt) {
    double b[5];
    host_gpu_check(hsmc_gpu_get_box(r->gpu, b), "get_box");
    r->in.rho = b[4];
    r->box.lx = b[0];
    r->box.ly = b[1];
    r->box.lz = b[2];
    r->box.vol = b[3];
  }
}
