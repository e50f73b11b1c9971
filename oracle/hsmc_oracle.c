/*
 * Oracle test infrastructure (not product code): CPU restatement of the HSMC
 * reference's local-move hard-sphere Monte Carlo path.  See hsmc_oracle.h.
 *
 * Every routine names the reference lines it follows (paths relative to the
 * reference project).  Floating-point expressions keep the reference's
 * operation order and are compiled with -ffp-contract=off, so results are
 * bit-identical to the reference built the same way.
 */
#include "hsmc_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "legendre.h"

/* ------------------------------------------------------------------ MT19937
 * GSL's mt19937 as used by src/rng.c:21-36: seed 0 -> 4357, Matsumoto &
 * Nishimura 2002 seeding, 32-bit tempered output, get_double = out/(2^32-1),
 * uniform_int(n) = out / floor((2^32-1)/n) with rejection of k >= n. */
typedef struct {
  uint32_t w[624];
  int pos;
} hso_mt;

static void mt_init(hso_mt *m, unsigned long seed) {
  if (seed == 0) seed = 4357;
  m->w[0] = (uint32_t)(seed & 0xffffffffUL);
  for (int i = 1; i < 624; i++) m->w[i] = 1812433253u * (m->w[i - 1] ^ (m->w[i - 1] >> 30)) + (uint32_t)i;
  m->pos = 624;
}

static uint32_t mt_u32(hso_mt *m) {
  if (m->pos >= 624) {
    for (int k = 0; k < 624; k++) {
      uint32_t y = (m->w[k] & 0x80000000u) | (m->w[(k + 1) % 624] & 0x7fffffffu);
      uint32_t v = m->w[(k + 397) % 624] ^ (y >> 1);
      m->w[k] = (y & 1u) ? (v ^ 0x9908b0dfu) : v;
    }
    m->pos = 0;
  }
  uint32_t y = m->w[m->pos++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

/* Draw source: the generator, or a scripted list of values (replay). */
typedef struct {
  const uint32_t *raw;
  size_t raw_n, raw_pos;
  const int *ints;
  size_t int_n, int_pos;
} hso_script;

/* Coefficients of the Grundke-Henderson cavity function over the
 * Verlet-Weis g(r) and the Percus-Yevick solution (src/analytic.c:23-31). */
typedef struct {
  double ay0, ay1, ay2, ay3;
  double AA, mu, etaW, dW;
  double complex t0, t1, t2, a00, a01, a02;
} hso_psi;

struct hso_sim {
  /* input (src/read_input.h:4-71 subset) */
  double rho;
  int nx, ny, nz, type;
  double neigh_dr;
  int max_part;
  double dr_max, dv_max, press;
  /* box (src/sim_info.h:11-18) */
  double lx, ly, lz, vol, cell_size;
  int n, per_cell;
  double (*conf)[4];
  /* cell list (src/cell_list.h:6-19); table row = [count, ids...] */
  int num_x, num_y, num_z, num_tot;
  double size_x, size_y, size_z;
  int *table;
  int neigh[27];
  int *neigh_mat;
  /* generator */
  hso_mt mt;
  hso_script script;
  /* counters (src/moves.c:22-24), kept 64-bit */
  unsigned long long moves, acc, rej, vmoves, vacc, vrej;
  /* persistent observable state (file statics of the reference) */
  double pressv_rmax;
  /* cavity sampling (src/read_input.c:82-86) and its potential */
  double pcav, cav_min, cav_max;
  hso_psi psi;
  int err;
};

static double draw_double(hso_sim *s) {
  uint32_t r;
  if (s->script.raw) {
    if (s->script.raw_pos >= s->script.raw_n) {
      s->err = HSO_ERR_ARG;
      return 0.5;
    }
    r = s->script.raw[s->script.raw_pos++];
  } else {
    r = mt_u32(&s->mt);
  }
  return (double)r / (double)4294967295u; /* src/rng.c:29-31 */
}

static int draw_int(hso_sim *s, int range) {
  if (s->script.ints) {
    if (s->script.int_pos >= s->script.int_n) {
      s->err = HSO_ERR_ARG;
      return 0;
    }
    int v = s->script.ints[s->script.int_pos++];
    if (v < 0 || v >= range) {
      s->err = HSO_ERR_ARG;
      return 0;
    }
    return v;
  }
  uint32_t bucket = 4294967295u / (uint32_t)range, k; /* src/rng.c:34-36 */
  do {
    k = mt_u32(&s->mt) / bucket;
  } while (k >= (uint32_t)range);
  return (int)k;
}

static void script_set(hso_sim *s, const uint32_t *raw, size_t nraw, const int *ints, size_t nint) {
  s->script.raw = raw;
  s->script.raw_n = nraw;
  s->script.raw_pos = 0;
  s->script.ints = ints;
  s->script.int_n = nint;
  s->script.int_pos = 0;
}

static void script_clear(hso_sim *s) { script_set(s, NULL, 0, NULL, 0); }

void hso_rng_raw(unsigned long seed, int n, uint32_t *out) {
  hso_mt m;
  mt_init(&m, seed);
  for (int i = 0; i < n; i++) out[i] = mt_u32(&m);
}

void hso_rng_uniform_int(unsigned long seed, unsigned long range, int n, int *out) {
  hso_sim tmp;
  memset(&tmp, 0, sizeof(tmp));
  mt_init(&tmp.mt, seed);
  for (int i = 0; i < n; i++) out[i] = draw_int(&tmp, (int)range);
}

/* ---------------------------------------------------------------- box/init */

/* src/sim_info.c:32-71 */
static void box_init(hso_sim *s) {
  int per_cell = (s->type == 1) ? 1 : 4;
  double cell_vol = per_cell / s->rho;
  double cell_size = pow(cell_vol, 1. / 3.);
  s->lx = s->nx * cell_size;
  s->ly = s->ny * cell_size;
  s->lz = s->nz * cell_size;
  s->vol = s->nx * s->ny * s->nz * cell_vol;
  s->cell_size = cell_size;
  s->per_cell = per_cell;
}

/* src/sim_info.c:120-156 */
static int lattice_init(hso_sim *s) {
  double a = s->cell_size;
  int id = 0;
  if (s->type == 1) {
    if (a < 1) return HSO_ERR_INIT_OVERLAP;
    for (int i = 0; i < s->nx; i++)
      for (int j = 0; j < s->ny; j++)
        for (int k = 0; k < s->nz; k++) {
          double *p = s->conf[id];
          p[0] = id;
          p[1] = i * a;
          p[2] = j * a;
          p[3] = k * a;
          id++;
        }
  } else {
    if (a / sqrt(2.0) < 1) return HSO_ERR_INIT_OVERLAP;
    for (int i = 0; i < s->nx; i++)
      for (int j = 0; j < s->ny; j++)
        for (int k = 0; k < s->nz; k++) {
          double site[4][3] = {{i * a, j * a, k * a},
                               {(i + 0.5) * a, (j + 0.5) * a, k * a},
                               {(i + 0.5) * a, j * a, (k + 0.5) * a},
                               {i * a, (j + 0.5) * a, (k + 0.5) * a}};
          for (int q = 0; q < 4; q++) {
            s->conf[id][0] = id;
            s->conf[id][1] = site[q][0];
            s->conf[id][2] = site[q][1];
            s->conf[id][3] = site[q][2];
            id++;
          }
        }
  }
  return HSO_OK;
}

/* --------------------------------------------------------------- cell list */

/* src/cell_list.c:237-246 (the x stride is num_x*num_x, as in the reference) */
static int cell_index_of(const hso_sim *s, double x, double y, double z) {
  return (int)(x / s->size_x) * s->num_x * s->num_x + (int)(y / s->size_y) * s->num_y + (int)(z / s->size_z);
}

static int cell_of_particle(const hso_sim *s, int id) {
  return cell_index_of(s, s->conf[id][1], s->conf[id][2], s->conf[id][3]);
}

/* src/cell_list.c:92-131; when fewer than 27 cells fit, three per axis are
 * used (the reference leaves its total unchanged there; it is kept
 * consistent here). */
static int cell_geometry(hso_sim *s, int init) {
  if (init) {
    s->num_x = (int)floor(s->lx / s->neigh_dr);
    s->num_y = (int)floor(s->ly / s->neigh_dr);
    s->num_z = (int)floor(s->lz / s->neigh_dr);
    s->num_tot = s->num_x * s->num_y * s->num_z;
    if (s->num_tot < 27) {
      s->num_x = s->num_y = s->num_z = 3;
      s->num_tot = 27;
    }
  }
  s->size_x = s->lx / s->num_x;
  s->size_y = s->ly / s->num_y;
  s->size_z = s->lz / s->num_z;
  if (s->size_x < 1.0 || s->size_y < 1.0 || s->size_z < 1.0) return HSO_ERR_CELL_TOO_SMALL;
  return HSO_OK;
}

/* src/cell_list.c:253-301 */
static void neigh_table(hso_sim *s) {
  for (int a = 0; a < s->num_x; a++)
    for (int b = 0; b < s->num_y; b++)
      for (int c = 0; c < s->num_z; c++) {
        int ref = a * s->num_x * s->num_x + b * s->num_y + c;
        int q = 0;
        for (int i = -1; i < 2; i++)
          for (int j = -1; j < 2; j++)
            for (int k = -1; k < 2; k++) {
              int x = a + i, y = b + j, z = c + k;
              if (x > s->num_x - 1) x -= s->num_x;
              else if (x < 0) x += s->num_x;
              if (y > s->num_y - 1) y -= s->num_y;
              else if (y < 0) y += s->num_y;
              if (z > s->num_z - 1) z -= s->num_z;
              else if (z < 0) z += s->num_z;
              s->neigh_mat[ref * 27 + q++] = x * s->num_x * s->num_x + y * s->num_y + z;
            }
      }
}

static int *row(const hso_sim *s, int cell) { return s->table + (size_t)cell * s->max_part; }

/* src/cell_list.c:142-175 */
static int cell_rebuild(hso_sim *s) {
  int e = cell_geometry(s, 0);
  if (e) return e;
  for (int c = 0; c < s->num_tot; c++) {
    int *r = row(s, c);
    r[0] = 0;
    for (int j = 1; j < s->max_part; j++) r[j] = -1;
  }
  for (int i = 0; i < s->n; i++) {
    int c = cell_of_particle(s, i);
    if (c < 0 || c >= s->num_tot) return HSO_ERR_ARG;
    int *r = row(s, c);
    r[0] += 1;
    if (r[0] > s->max_part - 1) return HSO_ERR_CELL_OVERFLOW;
    r[r[0]] = i;
  }
  return HSO_OK;
}

/* src/cell_list.c:180-220: delete with shift, then append */
static int cell_move(hso_sim *s, int from, int to, int id) {
  int *r = row(s, from);
  int cnt = r[0], found = 0;
  for (int j = 1; j <= cnt; j++) {
    if (!found && r[j] == id) found = 1;
    if (found) r[j] = (j < cnt) ? r[j + 1] : -1;
  }
  if (!found) return HSO_ERR_CELL_DELETE;
  r[0] = cnt - 1;
  int *t = row(s, to);
  t[0] += 1;
  if (t[0] > s->max_part - 1) return HSO_ERR_CELL_OVERFLOW;
  t[t[0]] = id;
  return HSO_OK;
}

/* ------------------------------------------------------------ distances */

/* src/moves.c:400-431 (the value compared against 1.0 by every caller) */
static double pair_dist(const hso_sim *s, const double *a, const double *b, double sf) {
  double lx = s->lx * sf, ly = s->ly * sf, lz = s->lz * sf;
  double hx = lx / 2.0, hy = ly / 2.0, hz = lz / 2.0;
  double dx = (a[1] - b[1]) * sf;
  double dy = (a[2] - b[2]) * sf;
  double dz = (a[3] - b[3]) * sf;
  if (dx > hx) dx -= lx;
  else if (dx < -hx) dx += lx;
  if (dy > hy) dy -= ly;
  else if (dy < -hy) dy += ly;
  if (dz > hz) dz -= lz;
  else if (dz < -hz) dz += lz;
  return sqrt(dx * dx + dy * dy + dz * dz);
}

/* src/moves.c:157-212 */
static int overlap_of(const hso_sim *s, int id, double sf) {
  int c = cell_of_particle(s, id);
  if (c < 0 || c >= s->num_tot) return 0;
  const int *nb = s->neigh_mat + (size_t)c * 27;
  for (int q = 0; q < 27; q++) {
    const int *r = row(s, nb[q]);
    for (int j = 1; j <= r[0]; j++) {
      int other = r[j];
      double d = pair_dist(s, s->conf[id], s->conf[other], sf);
      if (d < 1.0 && other != id) return 1;
    }
  }
  return 0;
}

/* src/moves.c:215-226 */
static void wrap_into_box(const hso_sim *s, double *p) {
  if (p[1] > s->lx) p[1] -= s->lx;
  else if (p[1] < 0.0) p[1] += s->lx;
  if (p[2] > s->ly) p[2] -= s->ly;
  else if (p[2] < 0.0) p[2] += s->ly;
  if (p[3] > s->lz) p[3] -= s->lz;
  else if (p[3] < 0.0) p[3] += s->lz;
}

/* ------------------------------------------------------------------- moves */

/* src/moves.c:27-80 */
static int particle_move(hso_sim *s) {
  int id = draw_int(s, s->n);
  double ux = draw_double(s), uy = draw_double(s), uz = draw_double(s);
  double *p = s->conf[id];
  double ox = p[1], oy = p[2], oz = p[3];
  int c_old = cell_of_particle(s, id);
  p[1] += (ux - 0.5) * s->dr_max;
  p[2] += (uy - 0.5) * s->dr_max;
  p[3] += (uz - 0.5) * s->dr_max;
  wrap_into_box(s, p);
  int accepted = 0;
  if (overlap_of(s, id, 1.0)) {
    p[1] = ox;
    p[2] = oy;
    p[3] = oz;
    s->rej++;
  } else {
    int c_new = cell_of_particle(s, id);
    if (c_new != c_old) {
      int e = cell_move(s, c_old, c_new, id);
      if (e) s->err = e;
    }
    s->acc++;
    accepted = 1;
  }
  s->moves++;
  return accepted;
}

/* src/moves.c:83-153 */
static int volume_move(hso_sim *s) {
  double r_dv = draw_double(s);
  double log_vol_new = log(s->vol) + (r_dv - 0.5) * s->dv_max;
  double vol_new = exp(log_vol_new);
  double ratio = vol_new / s->vol;
  double sf = pow(ratio, 1. / 3.);
  int overlap = 0;
  for (int i = 0; i < s->n && !overlap; i++) overlap = overlap_of(s, i, sf);
  int accepted = 0;
  if (!overlap) {
    double boltz = exp(s->press * (s->vol - vol_new) + (s->n + 1) * log(ratio));
    double r_acc = draw_double(s);
    if (r_acc >= boltz) {
      s->vrej++;
    } else {
      s->vacc++;
      accepted = 1;
      s->rho = s->n / vol_new;
      box_init(s);
      for (int i = 0; i < s->n; i++) {
        s->conf[i][1] *= sf;
        s->conf[i][2] *= sf;
        s->conf[i][3] *= sf;
        wrap_into_box(s, s->conf[i]);
      }
      int e = cell_rebuild(s);
      if (e) s->err = e;
    }
  } else {
    s->vrej++;
  }
  s->vmoves++;
  return accepted;
}

/* ---------------------------------------------------------------- lifecycle */

hso_sim *hso_create(double rho, int nx, int ny, int nz, int type, double neigh_dr, int neigh_max_part,
                    double dr_max, double dv_max, double press, unsigned long seed, int *err) {
  int e = HSO_OK;
  hso_sim *s = (hso_sim *)calloc(1, sizeof(hso_sim));
  if (!s) {
    if (err) *err = HSO_ERR_ALLOC;
    return NULL;
  }
  s->rho = rho;
  s->nx = nx;
  s->ny = ny;
  s->nz = nz;
  s->type = type;
  s->neigh_dr = neigh_dr;
  s->max_part = neigh_max_part;
  s->dr_max = dr_max;
  s->dv_max = dv_max;
  s->press = press;
  s->pressv_rmax = 1.05; /* src/compute_press.c:36 */
  box_init(s);
  s->n = nx * ny * nz * s->per_cell;
  s->conf = malloc(sizeof(*s->conf) * (size_t)s->n);
  if (!s->conf) e = HSO_ERR_ALLOC;
  if (!e) e = lattice_init(s);
  mt_init(&s->mt, seed);
  if (!e) e = cell_geometry(s, 1);
  if (!e) {
    s->table = malloc(sizeof(int) * (size_t)s->num_tot * (size_t)s->max_part);
    s->neigh_mat = malloc(sizeof(int) * (size_t)s->num_tot * 27);
    if (!s->table || !s->neigh_mat) e = HSO_ERR_ALLOC;
  }
  if (!e) e = cell_rebuild(s);
  if (!e) neigh_table(s);
  if (e) {
    hso_destroy(s);
    if (err) *err = e;
    return NULL;
  }
  if (err) *err = HSO_OK;
  return s;
}

void hso_destroy(hso_sim *s) {
  if (!s) return;
  free(s->conf);
  free(s->table);
  free(s->neigh_mat);
  free(s);
}

int hso_n(const hso_sim *s) { return s->n; }
int hso_last_error(const hso_sim *s) { return s->err; }

void hso_box(const hso_sim *s, double *out) {
  out[0] = s->lx;
  out[1] = s->ly;
  out[2] = s->lz;
  out[3] = s->vol;
  out[4] = s->rho;
  out[5] = s->size_x;
  out[6] = (double)s->num_x;
  out[7] = s->dr_max;
  out[8] = s->dv_max;
}

void hso_get_config(const hso_sim *s, double *out) { memcpy(out, s->conf, sizeof(double) * 4 * (size_t)s->n); }

int hso_set_config(hso_sim *s, const double *in) {
  memcpy(s->conf, in, sizeof(double) * 4 * (size_t)s->n);
  return cell_rebuild(s);
}

/* Lattice restart after the optimiser (src/nvt.c:58-62). */
int hso_reset_lattice(hso_sim *s) {
  int e = lattice_init(s);
  if (e) return e;
  e = cell_geometry(s, 1);
  if (e) return e;
  e = cell_rebuild(s);
  if (!e) neigh_table(s);
  return e;
}

void hso_set_steps(hso_sim *s, double dr_max, double dv_max) {
  s->dr_max = dr_max;
  s->dv_max = dv_max;
}

void hso_counters(const hso_sim *s, unsigned long long *out) {
  out[0] = s->moves;
  out[1] = s->acc;
  out[2] = s->rej;
  out[3] = s->vmoves;
  out[4] = s->vacc;
  out[5] = s->vrej;
}

void hso_reset_counters(hso_sim *s) { s->moves = s->acc = s->rej = s->vmoves = s->vacc = s->vrej = 0; }

/* ------------------------------------------------------------------ sweeps */

/* src/nvt.c:201-209 */
int hso_sweeps_nvt(hso_sim *s, int n) {
  for (int k = 0; k < n && !s->err; k++)
    for (int i = 0; i < s->n; i++) particle_move(s);
  return s->err;
}

/* src/npt.c:177-196 */
int hso_sweeps_npt(hso_sim *s, int n) {
  for (int k = 0; k < n && !s->err; k++)
    for (int i = 0; i < s->n; i++) {
      if (draw_int(s, s->n + 1) < s->n) particle_move(s);
      else volume_move(s);
    }
  return s->err;
}

/* ------------------------------------------------------ cavity potential */

/* coeff_py (src/analytic.c:174-230) */
static void psi_coeff_py(hso_psi *c, double eta) {
  double complex eta2 = eta * eta;
  double complex ometa = 1.0 - eta, ometa2 = ometa * ometa;
  double complex opeta_2 = 1.0 + eta / 2.0;
  double complex op2eta = 1.0 + 2 * eta;
  double complex ff = 3.0 + 3. * eta - eta2;
  double complex eta2_ff2 = (eta2 / ff) * (eta2 / ff);
  double complex tetaff = cpow(2 * eta * ff, 1. / 3.);
  double complex yp = cpow(sqrt(1. + 2. * eta2_ff2) + 1., 1. / 3.);
  double complex ym = -cpow(sqrt(1. + 2. * eta2_ff2) - 1., 1. / 3.);
  double complex jj = cexp((2. / 3.) * M_PI * I);
  double complex jj1 = jj;
  double complex jjm1 = 1. / jj1;
  double complex jj2 = jj * jj;
  double complex jjm2 = 1. / jj2;
  c->t0 = (-2 * eta + tetaff * (yp + ym)) / ometa;
  c->t1 = (-2 * eta + tetaff * (yp * jj1 + ym * jjm1)) / ometa;
  c->t2 = (-2 * eta + tetaff * (yp * jj2 + ym * jjm2)) / ometa;
  double complex L0 = opeta_2 * c->t0 + op2eta;
  double complex L1 = opeta_2 * c->t1 + op2eta;
  double complex L2 = opeta_2 * c->t2 + op2eta;
  double complex S10 = 3 * ometa2 * c->t0 * c->t0 + 12. * eta * ometa * c->t0 + 18. * eta2;
  double complex S11 = 3 * ometa2 * c->t1 * c->t1 + 12. * eta * ometa * c->t1 + 18. * eta2;
  double complex S12 = 3 * ometa2 * c->t2 * c->t2 + 12. * eta * ometa * c->t2 + 18. * eta2;
  c->a00 = c->t0 * L0 / S10;
  c->a01 = c->t1 * L1 / S11;
  c->a02 = c->t2 * L2 / S12;
}

/* rdf_py (src/analytic.c:143-170) */
static double psi_rdf_py(const hso_psi *c, double xx, double sigma) {
  double complex xx_hs = xx / sigma;
  if (creal(xx_hs) < 1.0) return 0.0;
  double complex g1 = c->a00 * cexp(c->t0 * (xx_hs - 1)) + c->a01 * cexp(c->t1 * (xx_hs - 1)) +
                      c->a02 * cexp(c->t2 * (xx_hs - 1));
  return creal(g1) / creal(xx_hs);
}

/* coeff_vw (src/analytic.c:103-140) */
static void psi_coeff_vw(hso_psi *c, double eta) {
  double eta2 = eta * eta;
  double eta3 = eta2 * eta, eta4 = eta2 * eta2;
  double ometa = 1. - eta, ometa3 = ometa * ometa * ometa;
  double ometa4 = ometa3 * ometa;
  double zz_cs = (1 + eta + eta2 - eta3) / ometa3;
  double mu_cs = ometa4 / (1 + 4. * eta + 4. * eta2 - 4. * eta3 + eta4);
  c->dW = pow(1 - eta / 16., 1. / 3.);
  double dW3 = c->dW * c->dW * c->dW, dW4 = dW3 * c->dW;
  c->etaW = eta * dW3;
  double op2etaW2 = (1 + 2 * c->etaW) * (1 + 2 * c->etaW);
  double ometaW = 1. - c->etaW;
  double ometaW3 = ometaW * ometaW * ometaW;
  double ometaW4 = ometaW3 * ometaW;
  double mu_py = ometaW4 / op2etaW2;
  psi_coeff_py(c, c->etaW);
  c->AA = (zz_cs - 1.0) / (4.0 * eta) - psi_rdf_py(c, 1.0, c->dW);
  c->mu = 12 * c->AA * eta /
          (mu_cs - mu_py +
           (c->etaW * (27.0 * c->etaW * (1 + c->etaW) - 8.0 * c->dW * op2etaW2 +
                       dW4 * (8.0 + 5.0 * c->etaW + 5.0 * c->etaW * c->etaW))) /
               (dW4 * (-ometaW3)));
}

/* rdf_vw (src/analytic.c:79-99) */
static double psi_rdf_vw(const hso_psi *c, double xx, double sigma) {
  double xx_hs = xx / sigma;
  if (xx_hs < 1.0) return 0.0;
  double delta_g1 = (c->AA / xx_hs) * exp(-c->mu * (xx_hs - 1)) * cos(c->mu * (xx_hs - 1));
  return psi_rdf_py(c, xx_hs, c->dW) + delta_g1;
}

/* coeff_gh (src/analytic.c:57-75) */
static void psi_coeff_gh(hso_psi *c, double eta) {
  psi_coeff_vw(c, eta);
  double eta2 = eta * eta, eta3 = eta2 * eta;
  double ometa = 1. - eta, ometa3 = ometa * ometa * ometa;
  double ometaW = 1. - c->etaW, ometaW3 = ometaW * ometaW * ometaW;
  double g1 = psi_rdf_py(c, 1.0, c->dW) + c->AA;
  double dg1 = -(9. / 2.) * c->etaW * (1 + c->etaW) / ometaW3 - c->AA * (1 + c->mu);
  c->ay0 = (8. * eta - 9. * eta2 + 3. * eta3) / ometa3;
  c->ay1 = -3. * eta * (2. - eta) / ometa3;
  c->ay2 = -(dg1 / g1) - 3. * c->ay0 - 2. * c->ay1 + 3. * log(g1);
  c->ay3 = 1. / 3. * ((dg1 / g1) - c->ay1 - 2. * c->ay2);
}

/* lny_gh (src/analytic.c:34-54) with sigma = 1 */
static double psi_lny(const hso_psi *c, double xx) {
  double xx_hs = xx / 1.0;
  if (xx_hs < 1.0) return c->ay0 + c->ay1 * xx_hs + c->ay2 * xx_hs * xx_hs + c->ay3 * xx_hs * xx_hs * xx_hs;
  return log(psi_rdf_vw(c, xx, 1.0));
}

/* The cavity interaction psi(x) = ln y_GH(x) at packing fraction pi rho / 6
 * (cavity_interaction, src/moves.c:434-440), for n distances. */
void hso_cavity_psi(double rho, int n, const double *x, double *out) {
  hso_psi c;
  psi_coeff_gh(&c, M_PI * rho / 6.0);
  for (int k = 0; k < n; k++) out[k] = psi_lny(&c, x[k]);
}

/* The coefficients in the order ay0..ay3, AA, mu, etaW, dW, then the real
 * and imaginary parts of t0, t1, t2, a00, a01, a02 (20 doubles). */
void hso_cavity_coeffs(double rho, double *out) {
  hso_psi c;
  psi_coeff_gh(&c, M_PI * rho / 6.0);
  const double v[8] = {c.ay0, c.ay1, c.ay2, c.ay3, c.AA, c.mu, c.etaW, c.dW};
  const double complex z[6] = {c.t0, c.t1, c.t2, c.a00, c.a01, c.a02};
  for (int k = 0; k < 8; k++) out[k] = v[k];
  for (int k = 0; k < 6; k++) {
    out[8 + 2 * k] = creal(z[k]);
    out[9 + 2 * k] = cimag(z[k]);
  }
}

/* ---------------------------------------------------------- cavity moves */

/* cavity_set_distance (src/cavity_nvt.c:172-186): cavity 1 on cavity 0,
 * shifted along z by the middle of the allowed range. */
int hso_cavity_setup(hso_sim *s, double pcav, double maxdr, double mindr) {
  s->pcav = pcav;
  s->cav_max = maxdr;
  s->cav_min = mindr;
  psi_coeff_gh(&s->psi, M_PI * s->rho / 6.0);
  double ave = (maxdr + mindr) / 2.0;
  s->conf[1][1] = s->conf[0][1];
  s->conf[1][2] = s->conf[0][2];
  s->conf[1][3] = s->conf[0][3] + ave;
  if (s->conf[1][3] > s->lz) s->conf[1][3] -= s->lz;
  else if (s->conf[1][3] < 0.0) s->conf[1][3] += s->lz;
  return cell_rebuild(s);
}

/* cavity_check_move (src/moves.c:333-396) after the proposal; returns 0 to
 * accept, 1 when the cavities leave the allowed range, 2 when the Metropolis
 * test fails, 3 on an overlap.  u_acc < 0 draws the uniform. */
static int cavity_decide(hso_sim *s, int id, int type, double en_old, double u_acc) {
  if (type == 1) {
    double d = pair_dist(s, s->conf[0], s->conf[1], 1.0);
    if (d < s->cav_min || d > s->cav_max) return 1;
    double boltz = exp(-(psi_lny(&s->psi, d) - en_old));
    double r = u_acc < 0 ? draw_double(s) : u_acc;
    if (r > boltz) return 2;
  }
  int c = cell_of_particle(s, id);
  if (c < 0 || c >= s->num_tot) return 3;
  const int *nb = s->neigh_mat + (size_t)c * 27;
  for (int q = 0; q < 27; q++) {
    const int *r = row(s, nb[q]);
    for (int j = 1; j <= r[0]; j++) {
      int other = r[j];
      double d = pair_dist(s, s->conf[id], s->conf[other], 1.0);
      if (type == 0 && other != id && d < 1.0) return 3;
      if (type == 1 && other >= 2 && d < 1.0) return 3;
    }
  }
  return 0;
}

/* cavity_part_move (src/moves.c:254-330) given the particle, its type and
 * the three step factors t = u - 0.5; u_acc < 0 draws the uniform. */
static int cavity_move_with(hso_sim *s, int id, int type, const double *t, double u_acc) {
  double *p = s->conf[id];
  double ox = p[1], oy = p[2], oz = p[3];
  int c_old = cell_of_particle(s, id);
  double en_old = 0.0;
  if (type == 1) {
    double d = pair_dist(s, s->conf[0], s->conf[1], 1.0);
    if (d < s->cav_min || d > s->cav_max) {
      s->err = HSO_ERR_ARG;
      return -1;
    }
    en_old = psi_lny(&s->psi, d);
  }
  p[1] += t[0] * s->dr_max;
  p[2] += t[1] * s->dr_max;
  p[3] += t[2] * s->dr_max;
  wrap_into_box(s, p);
  int dec = cavity_decide(s, id, type, en_old, u_acc);
  if (dec == 0) {
    int c_new = cell_of_particle(s, id);
    if (c_new != c_old) {
      int e = cell_move(s, c_old, c_new, id);
      if (e) s->err = e;
    }
    s->acc++;
  } else {
    p[1] = ox;
    p[2] = oy;
    p[3] = oz;
    s->rej++;
  }
  s->moves++;
  return dec;
}

/* cavity_sweep_nvt (src/cavity_nvt.c:161-169): N trials with the
 * reference's draws. */
int hso_cavity_sweeps(hso_sim *s, int n) {
  for (int k = 0; k < n && !s->err; k++)
    for (int i = 0; i < s->n && !s->err; i++) {
      double r_type = draw_double(s);
      int id, type;
      if (r_type > s->pcav) {
        id = draw_int(s, s->n - 2) + 2;
        type = 0;
      } else {
        id = draw_int(s, 2);
        type = 1;
      }
      double t[3];
      for (int d = 0; d < 3; d++) t[d] = draw_double(s) - 0.5;
      cavity_move_with(s, id, type, t, -1.0);
    }
  return s->err;
}

/* Cavity moves made by the device: cavity which[k] stepped by
 * (2r - 2^32 + 1) * 2^-33 * dr_max per axis (r = raw[3k..3k+2]) and tested
 * against the uniform (2 uacc[k] + 1) * 2^-33.  decision[k] as
 * cavity_decide. */
int hso_cavity_replay(hso_sim *s, int n, const int *which, const uint32_t *raw, const uint32_t *uacc,
                      int *decision) {
  for (int k = 0; k < n && !s->err; k++) {
    if (which[k] < 0 || which[k] > 1) return HSO_ERR_ARG;
    double t[3];
    for (int d = 0; d < 3; d++) t[d] = ldexp(2.0 * (double)raw[3 * k + d] - 4294967295.0, -33);
    double u = ldexp(2.0 * (double)uacc[k] + 1.0, -33);
    decision[k] = cavity_move_with(s, which[k], 1, t, u);
  }
  return s->err;
}

/* ----------------------------------------------------------- cluster moves */

/* rotate (src/cluster_nvt.c:342-365): point (xx, yy, zz) about the line
 * through (aa, bb, cc) with direction (uu, vv, ww) by theta. */
static void cluster_rotate(double xx, double yy, double zz, double aa, double bb, double cc, double uu, double vv,
                           double ww, double theta, double *xr, double *yr, double *zr) {
  double cost = cos(theta), sint = sin(theta);
  double uu2 = uu * uu, vv2 = vv * vv, ww2 = ww * ww;
  *xr = (aa * (vv2 + ww2) - uu * (bb * vv + cc * ww - uu * xx - vv * yy - ww * zz)) * (1 - cost) + xx * cost +
        (-cc * vv + bb * ww - ww * yy + vv * zz) * sint;
  *yr = (bb * (uu2 + ww2) - vv * (aa * uu + cc * ww - uu * xx - vv * yy - ww * zz)) * (1 - cost) + yy * cost +
        (cc * uu - aa * ww + ww * xx - uu * zz) * sint;
  *zr = (cc * (uu2 + vv2) - ww * (aa * uu + bb * vv - uu * xx - vv * yy - ww * zz)) * (1 - cost) + zz * cost +
        (-bb * uu + aa * vv - vv * xx + uu * yy) * sint;
}

/* cluster_move_part (src/cluster_nvt.c:312-339): rotate by pi, wrap, and
 * follow the particle in the cell list. */
static void cluster_move_one(hso_sim *s, int id, const double *piv, const double *axis) {
  double *p = s->conf[id];
  int c_old = cell_of_particle(s, id);
  cluster_rotate(p[1], p[2], p[3], piv[0], piv[1], piv[2], axis[0], axis[1], axis[2], M_PI, &p[1], &p[2], &p[3]);
  wrap_into_box(s, p);
  int c_new = cell_of_particle(s, id);
  if (c_new != c_old) {
    int e = cell_move(s, c_old, c_new, id);
    if (e) s->err = e;
  }
}

/* pocket_add (src/cluster_nvt.c:369-410): every particle of the 27 cells
 * around the moved one that it overlaps joins the pocket once. */
static void pocket_grow(hso_sim *s, int id, int *pocket, int *count) {
  int c = cell_of_particle(s, id);
  if (c < 0 || c >= s->num_tot) {
    s->err = HSO_ERR_ARG;
    return;
  }
  const int *nb = s->neigh_mat + (size_t)c * 27;
  for (int q = 0; q < 27; q++) {
    const int *r = row(s, nb[q]);
    for (int j = 1; j <= r[0]; j++) {
      int other = r[j];
      double d = pair_dist(s, s->conf[id], s->conf[other], 1.0);
      if (d < 1.0 && other != id) {
        int seen = 0;
        for (int k = 0; k < *count; k++) seen |= pocket[k] == other;
        if (!seen) pocket[(*count)++] = other;
      }
    }
  }
}

/* cluster_move (src/cluster_nvt.c:232-310) after its draws: move the seed,
 * then empty the pocket in random order (pocket_del keeps the survivors in
 * order, src/cluster_nvt.c:412-431). */
static int cluster_grow(hso_sim *s, const double *piv, int axis_id, int seed_id) {
  double axis[3] = {0.0, 0.0, 0.0};
  axis[axis_id] = 1.0;
  int *pocket = malloc(sizeof(int) * (size_t)s->n);
  if (!pocket) {
    s->err = HSO_ERR_ALLOC;
    return -1;
  }
  int count = 0, size = 1;
  cluster_move_one(s, seed_id, piv, axis);
  pocket_grow(s, seed_id, pocket, &count);
  while (count > 0 && !s->err) {
    int k = draw_int(s, count);
    int id = pocket[k];
    cluster_move_one(s, id, piv, axis);
    memmove(pocket + k, pocket + k + 1, sizeof(int) * (size_t)(count - k - 1));
    count--;
    pocket_grow(s, id, pocket, &count);
    size++;
  }
  free(pocket);
  return size;
}

/* One cluster move with the given pivot, axis (0, 1, 2 = x, y, z) and seed
 * particle; the pocket order still comes from the generator. */
int hso_cluster_move_at(hso_sim *s, const double *pivot, int axis, int seed_id, int *size) {
  if (axis < 0 || axis > 2 || seed_id < 0 || seed_id >= s->n) return HSO_ERR_ARG;
  int k = cluster_grow(s, pivot, axis, seed_id);
  if (size) *size = k;
  return s->err;
}

/* cluster_sweep_nvt (src/cluster_nvt.c:221-228) for n moves with the
 * reference's draws: pivot u * L per axis, axis rng_get_int(3), seed
 * rng_get_int(N). */
int hso_cluster_moves(hso_sim *s, int n, int *sizes) {
  for (int m = 0; m < n && !s->err; m++) {
    double piv[3];
    piv[0] = draw_double(s) * s->lx;
    piv[1] = draw_double(s) * s->ly;
    piv[2] = draw_double(s) * s->lz;
    int axis = draw_int(s, 3);
    int seed_id = draw_int(s, s->n);
    int k = cluster_grow(s, piv, axis, seed_id);
    if (sizes) sizes[m] = k;
  }
  return s->err;
}

/* part_move (src/moves.c:27-80) with u - 0.5 = (2r - 2^32 + 1) * 2^-33 per
 * axis, the step factor the GPU draws; the reference's own code forms the
 * same value from the draw 2r + 1 with maximum 2^33. */
int hso_replay_moves_offsets(hso_sim *s, int n, const int *ids, const uint32_t *raw, int *accepted) {
  for (int k = 0; k < n; k++) {
    int id = ids[k];
    if (id < 0 || id >= s->n) return HSO_ERR_ARG;
    double *p = s->conf[id];
    double ox = p[1], oy = p[2], oz = p[3];
    int c_old = cell_of_particle(s, id);
    for (int d = 0; d < 3; d++) {
      double t = (double)(2 * (long long)raw[3 * k + d] - 4294967295LL) * 0x1p-33;
      p[1 + d] += t * s->dr_max;
    }
    wrap_into_box(s, p);
    accepted[k] = 0;
    if (overlap_of(s, id, 1.0)) {
      p[1] = ox;
      p[2] = oy;
      p[3] = oz;
      s->rej++;
    } else {
      int c_new = cell_of_particle(s, id);
      if (c_new != c_old) {
        int e = cell_move(s, c_old, c_new, id);
        if (e) return e;
      }
      s->acc++;
      accepted[k] = 1;
    }
    s->moves++;
  }
  return s->err;
}

int hso_replay_moves(hso_sim *s, int n, const int *ids, const uint32_t *raw, int *accepted) {
  script_set(s, raw, 3 * (size_t)n, ids, (size_t)n);
  for (int k = 0; k < n; k++) accepted[k] = particle_move(s);
  script_clear(s);
  return s->err;
}

int hso_check_overlap_at(hso_sim *s, int i, double x, double y, double z) {
  double *p = s->conf[i];
  double ox = p[1], oy = p[2], oz = p[3];
  p[1] = x;
  p[2] = y;
  p[3] = z;
  int ov = overlap_of(s, i, 1.0);
  p[1] = ox;
  p[2] = oy;
  p[3] = oz;
  return ov;
}

int hso_scan_overlap(hso_sim *s, double sf) {
  for (int i = 0; i < s->n; i++)
    if (overlap_of(s, i, sf)) return 1;
  return 0;
}

int hso_vol_move_replay(hso_sim *s, const uint32_t *raw, int n_raw) {
  script_set(s, raw, (size_t)n_raw, NULL, 0);
  int a = volume_move(s);
  script_clear(s);
  return a;
}

/* ------------------------------------------------------------- observables */

/* src/compute_rdf.c:36-128 (cutoff limited to half the largest side, as the
 * reference's "minimum" check actually compares against the largest). */
int hso_rdf_counts(hso_sim *s, double dr, double rmax, double *out, int max_bins, double *rmax_used) {
  double side = s->lx;
  if (side < s->ly) side = s->ly;
  if (side < s->lz) side = s->lz;
  if (side < 2.0 * rmax) rmax = side / 2.0;
  int nb = (int)((rmax - 1.0) / dr);
  if (nb > max_bins || nb < 0) return -1;
  rmax = dr * nb + 1.0;
  for (int b = 0; b < nb; b++) out[b] = 0.0;
  for (int i = 0; i < s->n; i++)
    for (int j = i + 1; j < s->n; j++) {
      double d = pair_dist(s, s->conf[i], s->conf[j], 1.0);
      if (d < rmax) out[(int)((d - 1.0) / dr)] += 2.0;
    }
  if (rmax_used) *rmax_used = rmax;
  return nb;
}

/* src/compute_press.c:47-165 */
int hso_pressv_counts(hso_sim *s, double dr, double *out, int max_bins, double *rmax_used) {
  int nb = (int)((s->pressv_rmax - 1.0) / dr);
  if (nb > max_bins || nb < 0) return -1;
  s->pressv_rmax = dr * nb + 1.0;
  for (int b = 0; b < nb; b++) out[b] = 0.0;
  for (int i = 0; i < s->n; i++) {
    const int *nbr = s->neigh_mat + (size_t)cell_of_particle(s, i) * 27;
    for (int q = 0; q < 27; q++) {
      const int *r = row(s, nbr[q]);
      for (int j = 1; j <= r[0]; j++) {
        int other = r[j];
        double d = pair_dist(s, s->conf[i], s->conf[other], 1.0);
        if (d < s->pressv_rmax && other > i) out[(int)((d - 1.0) / dr)] += 2.0;
      }
    }
  }
  if (rmax_used) *rmax_used = s->pressv_rmax;
  return nb;
}

/* src/compute_press.c:191-273 */
int hso_presst_counts(hso_sim *s, double dxi, double xi_max, double *out, int max_n) {
  int nn = (int)(xi_max / dxi);
  if (nn > max_n || nn < 0) return -1;
  for (int k = 0; k < nn; k++) {
    double xi = (k + 1) * dxi;
    double ratio = 1 - xi;
    double sf = pow(ratio, 1. / 3.);
    out[k] = hso_scan_overlap(s, sf) ? 0.0 : 1.0;
  }
  return nn;
}

int hso_presst_counts_sf(hso_sim *s, const double *sf, int n, double *out) {
  for (int k = 0; k < n; k++) out[k] = hso_scan_overlap(s, sf[k]) ? 0.0 : 1.0;
  return n;
}

/* src/compute_widom_chem_pot.c:73-160: one insertion test at (x,y,z). */
static int insertion_overlaps(const hso_sim *s, double x, double y, double z) {
  int c = (int)(x / s->size_x) * s->num_x * s->num_x + (int)(y / s->size_y) * s->num_y + (int)(z / s->size_z);
  if (c < 0 || c >= s->num_tot) return -1;
  const int *nb = s->neigh_mat + (size_t)c * 27;
  double hx = s->lx / 2.0, hy = s->ly / 2.0, hz = s->lz / 2.0;
  for (int q = 0; q < 27; q++) {
    const int *r = row(s, nb[q]);
    for (int j = 1; j <= r[0]; j++) {
      const double *p = s->conf[r[j]];
      double dx = x - p[1], dy = y - p[2], dz = z - p[3];
      if (dx > hx) dx -= s->lx;
      else if (dx < -hx) dx += s->lx;
      if (dy > hy) dy -= s->ly;
      else if (dy < -hy) dy += s->ly;
      if (dz > hz) dz -= s->lz;
      else if (dz < -hz) dz += s->lz;
      if (sqrt(dx * dx + dy * dy + dz * dz) < 1.0) return 1;
    }
  }
  return 0;
}

/* src/compute_widom_chem_pot.c:44-71 with scripted uniforms; returns the
 * number of insertions without overlap, or -1 for a point outside the cell
 * table (a draw of exactly 1.0, where the reference indexes past its table). */
int hso_widom(hso_sim *s, int n, const uint32_t *raw) { return hso_widom_decisions(s, n, raw, NULL); }

int hso_widom_decisions(hso_sim *s, int n, const uint32_t *raw, uint8_t *overlap) {
  if (raw) script_set(s, raw, 3 * (size_t)n, NULL, 0);
  int ok = 0;
  for (int k = 0; k < n; k++) {
    double x = draw_double(s) * s->lx;
    double y = draw_double(s) * s->ly;
    double z = draw_double(s) * s->lz;
    int ov = insertion_overlaps(s, x, y, z);
    if (ov < 0) {
      if (raw) script_clear(s);
      return -1;
    }
    if (overlap) overlap[k] = (uint8_t)ov;
    if (!ov) ok++;
  }
  if (raw) script_clear(s);
  return ok;
}

int hso_widom_rng(hso_sim *s, int n) { return hso_widom_decisions(s, n, NULL, NULL); }

int hso_widom_points(hso_sim *s, int n, const double *pts, uint8_t *overlap) {
  int ok = 0;
  for (int k = 0; k < n; k++) {
    int ov = insertion_overlaps(s, pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]);
    if (ov < 0) return -1;
    if (overlap) overlap[k] = (uint8_t)ov;
    if (!ov) ok++;
  }
  return ok;
}

/* src/compute_order_parameter.c:25-229 */
double hso_ql(hso_sim *s, int l, double rc, double *per_particle, double *rc_used) {
  double side = s->size_x;
  if (side < s->size_y) side = s->size_y;
  if (side < s->size_z) side = s->size_z;
  if (side < rc) rc = side;
  int tlp1 = 2 * l + 1;
  double *qlm2 = malloc(sizeof(double) * (size_t)tlp1);
  double hx = s->lx / 2.0, hy = s->ly / 2.0, hz = s->lz / 2.0;
  double mean = 0.0;
  for (int i = 0; i < s->n; i++) {
    const int *nb = s->neigh_mat + (size_t)cell_of_particle(s, i) * 27;
    for (int m = 0; m < l + 1; m++) {
      int bonds = 0;
      double re = 0., im = 0., re_m = 0., im_m = 0.;
      for (int q = 0; q < 27; q++) {
        const int *r = row(s, nb[q]);
        for (int j = 1; j <= r[0]; j++) {
          int other = r[j];
          double dx = s->conf[i][1] - s->conf[other][1];
          double dy = s->conf[i][2] - s->conf[other][2];
          double dz = s->conf[i][3] - s->conf[other][3];
          if (dx > hx) dx -= s->lx;
          else if (dx < -hx) dx += s->lx;
          if (dy > hy) dy -= s->ly;
          else if (dy < -hy) dy += s->ly;
          if (dz > hz) dz -= s->lz;
          else if (dz < -hz) dz += s->lz;
          double d = sqrt(dx * dx + dy * dy + dz * dz);
          if (other != i && d <= rc) {
            double phi = atan2(dy, dx);
            if (phi < 0) phi += 2. * M_PI;
            bonds++;
            double plm = hso_sph_plm(l, m, dz / d);
            re += plm * cos(m * phi);
            im += plm * sin(m * phi);
            if (m % 2 != 0) plm *= -1.0;
            re_m += plm * cos(-m * phi);
            im_m += plm * sin(-m * phi);
          }
        }
      }
      if (bonds != 0) {
        re /= bonds;
        im /= bonds;
        re_m /= bonds;
        im_m /= bonds;
      }
      qlm2[l + m] = re * re + im * im;
      qlm2[l - m] = re_m * re_m + im_m * im_m;
    }
    double q = 0.0;
    for (int k = 0; k < tlp1; k++) q += qlm2[k];
    q *= 4 * M_PI / tlp1;
    q = sqrt(q);
    if (per_particle) per_particle[i] = q;
    mean += q / s->n;
  }
  free(qlm2);
  if (rc_used) *rc_used = rc;
  return mean;
}

/* src/optimizer.c:23-78 */
static double sample_acceptance(hso_sim *s, int sweeps) {
  hso_reset_counters(s);
  hso_sweeps_nvt(s, sweeps);
  return (double)s->acc / ((double)s->moves);
}

int hso_opt_nvt(hso_sim *s, int opt_sweeps, int opt_samples, double target, double *dr_out, double *acc_out) {
  int per = opt_sweeps / opt_samples;
  double dr1 = s->dr_max, a1 = sample_acceptance(s, per);
  if (a1 > target) s->dr_max *= 2;
  else s->dr_max /= 2;
  double dr2 = s->dr_max, a2 = sample_acceptance(s, per);
  for (int k = 0; k < opt_samples; k++) {
    s->dr_max = dr2 - (a2 - target) * (dr2 - dr1) / (a2 - a1);
    if (s->dr_max > 1.0) {
      s->dr_max = 1.0;
    } else if (s->dr_max <= 0.0) {
      s->dr_max = -s->dr_max;
      if (s->dr_max > 1.0) s->dr_max = dr2 / 2;
    }
    dr1 = dr2;
    a1 = a2;
    dr2 = s->dr_max;
    a2 = sample_acceptance(s, per);
  }
  if (dr_out) *dr_out = s->dr_max;
  if (acc_out) *acc_out = a2;
  return s->err;
}

/* -------------------------------------------------------- grid-free checks */

static double free_dist(double lx, double ly, double lz, const double *a, double x, double y, double z) {
  double hx = lx / 2.0, hy = ly / 2.0, hz = lz / 2.0;
  double dx = x - a[1], dy = y - a[2], dz = z - a[3];
  if (dx > hx) dx -= lx;
  else if (dx < -hx) dx += lx;
  if (dy > hy) dy -= ly;
  else if (dy < -hy) dy += ly;
  if (dz > hz) dz -= lz;
  else if (dz < -hz) dz += lz;
  return sqrt(dx * dx + dy * dy + dz * dz);
}

int hso_brute_overlap(const double *conf, int n, double lx, double ly, double lz, int skip, double x, double y,
                      double z) {
  const double(*c)[4] = (const double(*)[4])conf;
  for (int j = 0; j < n; j++) {
    if (j == skip) continue;
    if (free_dist(lx, ly, lz, c[j], x, y, z) < 1.0) return 1;
  }
  return 0;
}

/* All-pairs histogram in the reference's g(r) arithmetic: every unordered
 * pair with r < rmax adds 2 to bin (int)((r-1)/dr). */
int hso_brute_pair_hist(const double *conf, int n, double lx, double ly, double lz, double dr, double rmax,
                        int nbins, unsigned long long *counts) {
  const double(*c)[4] = (const double(*)[4])conf;
  for (int b = 0; b < nbins; b++) counts[b] = 0;
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++) {
      double d = free_dist(lx, ly, lz, c[j], c[i][1], c[i][2], c[i][3]);
      if (d < rmax) {
        int b = (int)((d - 1.0) / dr);
        if (b < 0 || b >= nbins) return -1;
        counts[b] += 2;
      }
    }
  return 0;
}

/* ------------------------------------------------- checkerboard replay */

/* Cell coordinate of a single-precision position on a shifted periodic grid;
 * the same arithmetic the GPU sweep uses to assign and confine particles. */
uint32_t hso_cell_of32(float x32, float shift32, float len32, float inv_w32, int nc) {
  float t = x32 - shift32;
  if (t < 0.0f) t += len32;
  int i = (int)(t * inv_w32);
  if (i >= nc) i -= nc;
  if (i < 0) i = 0;
  return (uint32_t)i;
}

static uint32_t flat_cell32(const double *p, const float *sh, const int *nc, const float *len32,
                            const float *inv_w32) {
  uint32_t ix = hso_cell_of32((float)p[1], sh[0], len32[0], inv_w32[0], nc[0]);
  uint32_t iy = hso_cell_of32((float)p[2], sh[1], len32[1], inv_w32[1], nc[1]);
  uint32_t iz = hso_cell_of32((float)p[3], sh[2], len32[2], inv_w32[2], nc[2]);
  return ix + (uint32_t)nc[0] * (iy + (uint32_t)nc[1] * iz);
}

int hso_replay_checkerboard(hso_sim *s, int n, const int *ids, const uint32_t *raw, const uint32_t *cells,
                            const float *shift32, const int *nc, const float *len32, const float *inv_w32,
                            int *decision) {
  for (int k = 0; k < n; k++) {
    int id = ids[k];
    if (id < 0 || id >= s->n) return HSO_ERR_ARG;
    double *p = s->conf[id];
    const float *sh = shift32 + 3 * (size_t)k;
    s->moves++;
    if (flat_cell32(p, sh, nc, len32, inv_w32) != cells[k]) {
      decision[k] = 3;
      continue;
    }
    /* u - 0.5 for the draw r: (2r - 2^32 + 1) * 2^-33 (exact), the value the
     * reference's own part_move forms from the draw 2r + 1 with maximum 2^33 */
    double q[4] = {p[0], p[1], p[2], p[3]};
    for (int d = 0; d < 3; d++) {
      double t = (double)(2 * (long long)raw[3 * k + d] - 4294967295LL) * 0x1p-33;
      q[1 + d] += t * s->dr_max;
    }
    wrap_into_box(s, q);
    if (flat_cell32(q, sh, nc, len32, inv_w32) != cells[k]) {
      decision[k] = 2;
      s->rej++;
      continue;
    }
    int c_old = cell_of_particle(s, id);
    double ox = p[1], oy = p[2], oz = p[3];
    p[1] = q[1];
    p[2] = q[2];
    p[3] = q[3];
    if (overlap_of(s, id, 1.0)) {
      p[1] = ox;
      p[2] = oy;
      p[3] = oz;
      decision[k] = 1;
      s->rej++;
      continue;
    }
    int c_new = cell_of_particle(s, id);
    if (c_new != c_old) {
      int e = cell_move(s, c_old, c_new, id);
      if (e) return e;
    }
    decision[k] = 0;
    s->acc++;
  }
  return s->err;
}
