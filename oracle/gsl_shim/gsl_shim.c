/*
 * Oracle test infrastructure (not product code).
 *
 * Implements the GSL subset declared in gsl/gsl_rng.h and
 * gsl/gsl_sf_legendre.h so the unmodified HSMC reference sources compile and
 * run here.  See the headers for the conventions followed.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "gsl/gsl_rng.h"
#include "gsl/gsl_sf_legendre.h"

/* ---------------------------------------------------------------- MT19937 */

#define MT_N 624
#define MT_M 397

/* Layout mirrors what a restart file holds for this generator: the 624-word
 * state followed by the position index. */
typedef struct {
  unsigned long mt[MT_N];
  int mti;
} mt_state;

static void mt_seed(mt_state *s, unsigned long seed) {
  if (seed == 0) seed = 4357; /* GSL's documented default seed */
  s->mt[0] = seed & 0xffffffffUL;
  for (int i = 1; i < MT_N; i++) {
    unsigned long prev = s->mt[i - 1];
    s->mt[i] = (1812433253UL * (prev ^ (prev >> 30)) + (unsigned long)i) & 0xffffffffUL;
  }
  s->mti = MT_N;
}

static void mt_refill(mt_state *s) {
  const unsigned long upper = 0x80000000UL, lower = 0x7fffffffUL;
  const unsigned long matrix_a = 0x9908b0dfUL;
  for (int k = 0; k < MT_N; k++) {
    unsigned long y = (s->mt[k] & upper) | (s->mt[(k + 1) % MT_N] & lower);
    unsigned long v = s->mt[(k + MT_M) % MT_N] ^ (y >> 1);
    if (y & 1UL) v ^= matrix_a;
    s->mt[k] = v;
  }
  s->mti = 0;
}

static unsigned long mt_next(mt_state *s) {
  if (s->mti >= MT_N) mt_refill(s);
  unsigned long y = s->mt[s->mti++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680UL;
  y ^= (y << 15) & 0xefc60000UL;
  y ^= (y >> 18);
  return y & 0xffffffffUL;
}

static const gsl_rng_type mt_type = {"mt19937", 0xffffffffUL, 0UL, sizeof(mt_state)};
const gsl_rng_type *gsl_rng_mt19937 = &mt_type;

/* ---------------------------------------------------------------- script */

static const unsigned long *script_raw = NULL;
static size_t script_raw_n = 0, script_raw_pos = 0;
static const int *script_int = NULL;
static size_t script_int_n = 0, script_int_pos = 0;

void hsmc_shim_script_raw(const unsigned long *vals, size_t n) {
  script_raw = vals;
  script_raw_n = n;
  script_raw_pos = 0;
}

void hsmc_shim_script_int(const int *vals, size_t n) {
  script_int = vals;
  script_int_n = n;
  script_int_pos = 0;
}

void hsmc_shim_script_off(void) {
  script_raw = NULL;
  script_int = NULL;
  script_raw_n = script_int_n = 0;
  script_raw_pos = script_int_pos = 0;
}

size_t hsmc_shim_script_left_raw(void) { return script_raw ? script_raw_n - script_raw_pos : 0; }
size_t hsmc_shim_script_left_int(void) { return script_int ? script_int_n - script_int_pos : 0; }

/* ---------------------------------------------------------------- gsl_rng */

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) {
  gsl_rng *r = (gsl_rng *)malloc(sizeof(gsl_rng));
  if (!r) return NULL;
  r->type = T;
  r->state = calloc(1, T->size);
  if (!r->state) {
    free(r);
    return NULL;
  }
  mt_seed((mt_state *)r->state, 0);
  return r;
}

void gsl_rng_set(const gsl_rng *r, unsigned long int seed) { mt_seed((mt_state *)r->state, seed); }

unsigned long int gsl_rng_max(const gsl_rng *r) { return r->type->max; }
unsigned long int gsl_rng_min(const gsl_rng *r) { return r->type->min; }

unsigned long int gsl_rng_get(const gsl_rng *r) {
  if (script_raw) {
    if (script_raw_pos >= script_raw_n) {
      fprintf(stderr, "gsl shim: scripted raw draws exhausted\n");
      exit(EXIT_FAILURE);
    }
    return script_raw[script_raw_pos++];
  }
  return mt_next((mt_state *)r->state);
}

unsigned long int gsl_rng_uniform_int(const gsl_rng *r, unsigned long int n) {
  if (script_int) {
    if (script_int_pos >= script_int_n) {
      fprintf(stderr, "gsl shim: scripted integer draws exhausted\n");
      exit(EXIT_FAILURE);
    }
    int v = script_int[script_int_pos++];
    if (v < 0 || (unsigned long)v >= n) {
      fprintf(stderr, "gsl shim: scripted integer %d outside [0,%lu)\n", v, n);
      exit(EXIT_FAILURE);
    }
    return (unsigned long)v;
  }
  unsigned long range = r->type->max - r->type->min;
  if (n == 0 || n > range) {
    fprintf(stderr, "gsl shim: uniform_int range %lu invalid\n", n);
    exit(EXIT_FAILURE);
  }
  unsigned long bucket = range / n, k;
  do {
    k = (gsl_rng_get(r) - r->type->min) / bucket;
  } while (k >= n);
  return k;
}

void gsl_rng_free(gsl_rng *r) {
  if (!r) return;
  free(r->state);
  free(r);
}

int gsl_rng_fwrite(FILE *stream, const gsl_rng *r) {
  return fwrite(r->state, r->type->size, 1, stream) == 1 ? 0 : 1;
}

int gsl_rng_fread(FILE *stream, gsl_rng *r) {
  return fread(r->state, r->type->size, 1, stream) == 1 ? 0 : 1;
}

/* ------------------------------------------------------ Legendre (sphPlm) */

#include "../legendre.h"

double gsl_sf_legendre_sphPlm(const int l, int m, const double x) {
  if (m < 0 || l < m || x < -1.0 || x > 1.0) {
    fprintf(stderr, "gsl shim: sphPlm domain error l=%d m=%d x=%g\n", l, m, x);
    exit(EXIT_FAILURE);
  }
  return hso_sph_plm(l, m, x);
}
