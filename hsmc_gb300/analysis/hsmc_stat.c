/* hsmc_stat: the analysis step of HSMC in C, so that averages and their
 * errors can be formed without Python.  It reads the files the drop-in
 * program (and the reference) write and prints what the reference's analysis
 * modules print:
 *
 *   pressv      pressure_virial  (python/hsmc_pressure.py:11-41): per block of
 *               samples the averaged contact histogram, a least-squares line
 *               g(r) = b0 + b1 r, Z = 1 + (2 pi / 3) rho (b0 + b1); mean and
 *               jackknife error over blocks
 *   presst      pressure_thermo (python/hsmc_pressure.py:46-107): per block
 *               -ln of the averaged non-overlap fraction against xi (zero
 *               bins dropped), slope / N = excess pressure, P = rho (1 + p_ex)
 *   presst-npt  the same with the density of each sample from density.dat
 *   mu          hsmc_chem_pot.ave and .std (python/hsmc_chem_pot.py:14-60):
 *               rows with no accepted insertion dropped, mean mu, mean
 *               acceptance in percent, jackknife error of mu
 *   op          hsmc_op.ave and .std (python/hsmc_op.py:14-73): mean q_l and
 *               Flyvbjerg-Petersen blocking
 *   density     hsmc_density.ave and .std (python/hsmc_density.py:14-68)
 *
 * Blocking and jackknife follow python/hsmc_stat.py:6-137: population
 * standard deviations, std / sqrt(n - 1) per blocking level, the data cut to
 * the largest power of two, leave-one-out means scaled by sqrt(n - 1).
 *
 * Usage: hsmc_stat [-d dir] [-b samples_per_block] [-j] command ...
 *   -j uses the jackknife inside blocking (jk_flag of blocking_std). */
#include <errno.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef struct {
  char **line;
  int n;
} lines_t;

static void die(const char *msg, const char *what) {
  fprintf(stderr, "hsmc_stat: %s%s%s\n", msg, what ? " " : "", what ? what : "");
  exit(EXIT_FAILURE);
}

static lines_t read_lines(const char *dir, const char *name) {
  char path[4096];
  snprintf(path, sizeof(path), "%s/%s", dir, name);
  FILE *f = fopen(path, "r");
  if (!f) die("cannot open", path);
  lines_t L = {NULL, 0};
  int cap = 0;
  char buf[4096];
  while (fgets(buf, sizeof(buf), f)) {
    if (L.n == cap) {
      cap = cap ? 2 * cap : 256;
      L.line = realloc(L.line, sizeof(char *) * (size_t)cap);
      if (!L.line) die("out of memory", NULL);
    }
    L.line[L.n++] = strdup(buf);
  }
  fclose(f);
  return L;
}

static void free_lines(lines_t *L) {
  for (int i = 0; i < L->n; i++) free(L->line[i]);
  free(L->line);
}

/* Rows of whitespace-separated numbers, '#' lines skipped (np.loadtxt). */
static double *load_table(const char *dir, const char *name, int cols, int *rows) {
  lines_t L = read_lines(dir, name);
  double *v = malloc(sizeof(double) * (size_t)cols * (size_t)(L.n + 1));
  int r = 0;
  for (int i = 0; i < L.n; i++) {
    const char *p = L.line[i];
    while (*p == ' ' || *p == '\t') p++;
    if (*p == '#' || *p == '\n' || *p == '\0') continue;
    char *end;
    for (int c = 0; c < cols; c++) {
      errno = 0;
      v[(size_t)r * cols + c] = strtod(p, &end);
      if (end == p) die("bad number in", name);
      p = end;
    }
    r++;
  }
  free_lines(&L);
  *rows = r;
  return v;
}

static double mean(const double *x, int n) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s += x[i];
  return s / n;
}

/* np.std: population standard deviation */
static double pstd(const double *x, int n) {
  const double m = mean(x, n);
  double s = 0.0;
  for (int i = 0; i < n; i++) s += (x[i] - m) * (x[i] - m);
  return sqrt(s / n);
}

/* jackknife (python/hsmc_stat.py:118-137): leave-one-out means; their
 * population std times sqrt(n - 1). */
static void jackknife(const double *x, int n, double *ave, double *err) {
  double tot = 0.0;
  for (int i = 0; i < n; i++) tot += x[i];
  double *xi = malloc(sizeof(double) * (size_t)n);
  for (int i = 0; i < n; i++) xi[i] = (tot - x[i]) / (n - 1);
  *ave = mean(xi, n);
  *err = pstd(xi, n) * sqrt((double)(n - 1));
  free(xi);
}

/* blocking_std (python/hsmc_stat.py:6-43) with its printout. */
static void blocking(const double *data, int nn, int jk) {
  int maxp2 = 0;
  while ((1 << (maxp2 + 1)) <= nn) maxp2++;
  const int nn_max = 1 << maxp2;
  if (nn_max < nn) {
    printf("WARNING: Used %d samples out of %d for variance estimation\n", nn_max, nn);
    nn = nn_max;
  }
  double *d = malloc(sizeof(double) * (size_t)nn);
  memcpy(d, data, sizeof(double) * (size_t)nn);
  printf("Transformation, variance\n");
  for (int ii = 0; ii < maxp2 - 1; ii++) {
    double s;
    if (jk) {
      double a;
      jackknife(d, nn, &a, &s);
    } else {
      s = pstd(d, nn) / sqrt((double)(nn - 1));
    }
    printf("%d %.8f\n", ii, s);
    for (int k = 0; k < nn / 2; k++) d[k] = (d[2 * k] + d[2 * k + 1]) / 2.0;
    nn /= 2;
  }
  free(d);
}

/* Least-squares line y = b0 + b1 x (the linear curve_fit of data_fit). */
static int line_fit(const double *x, const double *y, int n, double *b0, double *b1) {
  if (n < 2) return 0;
  const double mx = mean(x, n), my = mean(y, n);
  double sxx = 0.0, sxy = 0.0;
  for (int i = 0; i < n; i++) {
    sxx += (x[i] - mx) * (x[i] - mx);
    sxy += (x[i] - mx) * (y[i] - my);
  }
  if (sxx == 0.0) return 0;
  *b1 = sxy / sxx;
  *b0 = my - *b1 * mx;
  return 1;
}

/* read_pressure_output (python/hsmc_pressure.py:111-209): samples of
 * `header` lines + n_bins rows, the sizes on line 3 of the file; averaged in
 * blocks of `block` samples and fitted.  Returns the number of fitted blocks
 * (blocks whose fit is undefined are dropped); coeff[2k], coeff[2k+1] = b0, b1. */
static int pressure_blocks(const char *dir, const char *name, int block, int thermo, double **coeff, double *vol,
                           double *n_part) {
  lines_t L = read_lines(dir, name);
  const int header = 7;
  if (L.n < 4) die("too short:", name);
  double nb_d;
  if (sscanf(L.line[3], "%lf %lf %lf", &nb_d, vol, n_part) != 3) die("bad sizes line in", name);
  const int n_bins = (int)nb_d;
  const int per_sample = n_bins + header, per_block = block * per_sample;
  const int n_blk = per_block > 0 ? L.n / per_block : 0;
  double *c = malloc(sizeof(double) * 2 * (size_t)(n_blk + 1));
  double *x = malloc(sizeof(double) * (size_t)n_bins), *y = malloc(sizeof(double) * (size_t)n_bins);
  int out = 0;
  for (int b = 0; b < n_blk; b++) {
    for (int j = 0; j < n_bins; j++) y[j] = 0.0;
    for (int s = 0; s < block; s++) {
      const int base = (b * block + s) * per_sample + header;
      for (int j = 0; j < n_bins; j++) {
        double r, h;
        if (sscanf(L.line[base + j], "%lf %lf", &r, &h) != 2) die("bad histogram row in", name);
        x[j] = r;
        y[j] += h / block;
      }
    }
    int m = 0;
    for (int j = 0; j < n_bins; j++) {
      if (thermo) {
        if (y[j] == 0.0) continue;  // indeterminate forms removed
        x[m] = x[j];
        y[m] = -log(y[j]);
      } else {
        x[m] = x[j];
        y[m] = y[j];
      }
      m++;
    }
    double b0, b1;
    if (!line_fit(x, y, m, &b0, &b1)) continue;
    c[2 * out] = b0;
    c[2 * out + 1] = b1;
    out++;
  }
  free(x);
  free(y);
  free_lines(&L);
  *coeff = c;
  return out;
}

static void cmd_pressv(const char *dir, int block) {
  double *c, vol, np;
  const int n = pressure_blocks(dir, "press_virial.dat", block, 0, &c, &vol, &np);
  if (n < 2) die("not enough samples in", "press_virial.dat");
  const double dens = np / vol;
  double *p = malloc(sizeof(double) * (size_t)n);
  for (int k = 0; k < n; k++) p[k] = 1.0 + (2.0 * M_PI / 3.0) * dens * (c[2 * k] + c[2 * k + 1]);
  double ja, js;
  jackknife(p, n, &ja, &js);
  const double ave = mean(p, n);
  printf("Pressure from virial calculations\n");
  printf("Samples, average (HS units), variance (HS units), average (ISO units), variance (HS units)\n");
  printf("%d %.8f %.8f %.8f %.8f\n", n, ave * dens, js * dens, ave, js);
  free(p);
  free(c);
}

static void cmd_presst(const char *dir, int block, int npt) {
  double *c, vol, np;
  const int n = pressure_blocks(dir, "press_thermo.dat", block, 1, &c, &vol, &np);
  if (n < 2) die("not enough samples in", "press_thermo.dat");
  double *dens = malloc(sizeof(double) * (size_t)n), *p = malloc(sizeof(double) * (size_t)n);
  int n_dens = n;
  if (npt) {
    /* density.dat: three header lines, one sample per line, averaged in the
     * same blocks (read_density_output, python/hsmc_pressure.py:228-285) */
    lines_t L = read_lines(dir, "density.dat");
    const int avail = (L.n - 3) / block;
    n_dens = avail < n ? avail : n;
    for (int k = 0; k < n_dens; k++) {
      double s = 0.0;
      for (int j = 0; j < block; j++) s += strtod(L.line[3 + k * block + j], NULL) / block;
      dens[k] = s;
    }
    free_lines(&L);
    if (n_dens < 2) die("not enough samples in", "density.dat");
  } else {
    for (int k = 0; k < n; k++) dens[k] = np / vol;
  }
  const int m = npt ? n_dens : n;
  for (int k = 0; k < m; k++) p[k] = dens[k] * (1.0 + c[2 * k + 1] / np);
  double ja, ps, ds = 0.0;
  jackknife(p, m, &ja, &ps);
  const double pa = mean(p, m), da = npt ? mean(dens, m) : np / vol;
  if (npt) jackknife(dens, m, &ja, &ds);
  printf("Pressure from thermodynamic calculations\n");
  printf("Samples, average (HS units), std. dev. (HS units), average (ISO units), std. dev. (ISO units)\n");
  printf("%d %.8f %.8f %.8f %.8f\n", m, pa, ps, pa / da, ps / da);
  if (npt) {
    printf("Density from thermodynamic calculations\n");
    printf("Samples, average (HS units), std. dev. (HS units)\n");
    printf("%d %.8f %.8f\n", m, da, ds);
  }
  free(dens);
  free(p);
  free(c);
}

static void cmd_mu(const char *dir) {
  int rows;
  double *t = load_table(dir, "chem_pot.dat", 2, &rows);
  double *mu = malloc(sizeof(double) * (size_t)(rows + 1)), *acc = malloc(sizeof(double) * (size_t)(rows + 1));
  int n = 0;
  for (int i = 0; i < rows; i++)
    if (t[2 * i + 1] > 0) {  // rows with no accepted insertion removed
      mu[n] = t[2 * i];
      acc[n] = t[2 * i + 1];
      n++;
    }
  if (n < 2) die("not enough samples in", "chem_pot.dat");
  double ja, js;
  jackknife(mu, n, &ja, &js);
  printf("Average chemical potential: %.8f\n", mean(mu, n));
  printf("Percentage of accepted moves: %.8f\n", mean(acc, n) * 100);
  printf("Standard deviation of chemical potential: %.8f\n", js);
  free(t);
  free(mu);
  free(acc);
}

static void cmd_series(const char *dir, const char *file, const char *label, int jk) {
  int rows;
  double *v = load_table(dir, file, 1, &rows);
  if (rows < 2) die("not enough samples in", file);
  printf("Average %s: %.8f\n", label, mean(v, rows));
  blocking(v, rows, jk);
  free(v);
}

int main(int argc, char **argv) {
  const char *dir = ".";
  int block = 1, jk = 0, opt;
  while ((opt = getopt(argc, argv, "d:b:j")) != -1) {
    switch (opt) {
      case 'd': dir = optarg; break;
      case 'b': block = atoi(optarg); break;
      case 'j': jk = 1; break;
      default:
        fprintf(stderr, "usage: hsmc_stat [-d dir] [-b samples_per_block] [-j] pressv|presst|presst-npt|mu|op|density ...\n");
        return EXIT_FAILURE;
    }
  }
  if (block < 1 || optind >= argc) {
    fprintf(stderr, "usage: hsmc_stat [-d dir] [-b samples_per_block] [-j] pressv|presst|presst-npt|mu|op|density ...\n");
    return EXIT_FAILURE;
  }
  for (int i = optind; i < argc; i++) {
    const char *c = argv[i];
    if (!strcmp(c, "pressv")) cmd_pressv(dir, block);
    else if (!strcmp(c, "presst")) cmd_presst(dir, block, 0);
    else if (!strcmp(c, "presst-npt")) cmd_presst(dir, block, 1);
    else if (!strcmp(c, "mu")) cmd_mu(dir);
    else if (!strcmp(c, "op")) cmd_series(dir, "order_param.dat", "order parameter", jk);
    else if (!strcmp(c, "density")) cmd_series(dir, "density.dat", "density", jk);
    else die("unknown command", c);
  }
  return EXIT_SUCCESS;
}
