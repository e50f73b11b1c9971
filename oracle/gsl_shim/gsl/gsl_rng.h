/*
 * Oracle test infrastructure (not product code).
 *
 * Minimal stand-in for the GNU Scientific Library's random-number interface,
 * covering exactly the calls the HSMC reference makes in src/rng.c:21-53
 * (gsl_rng_alloc(gsl_rng_mt19937), gsl_rng_set, gsl_rng_max, gsl_rng_get,
 * gsl_rng_uniform_int, gsl_rng_free, gsl_rng_fwrite, gsl_rng_fread).
 *
 * GSL is an un-vendored dependency of the reference with no pinned version
 * (src/Makefile:8 only adds an include path).  The generator restated here is
 * MT19937 (Matsumoto & Nishimura 1998, with their 2002 seeding), using GSL's
 * documented conventions: seed 0 means 4357, max = 2^32-1, min = 0, and
 * uniform_int(n) divides the range into n equal buckets and rejects the
 * remainder.
 *
 * A "script" mode is added for replay: when armed, gsl_rng_get and
 * gsl_rng_uniform_int pop caller-supplied values instead of drawing, so the
 * reference's own move code can be driven with proposals generated elsewhere.
 */
#ifndef HSMC_ORACLE_GSL_RNG_H
#define HSMC_ORACLE_GSL_RNG_H

#include <stddef.h>
#include <stdio.h>

typedef struct {
  const char *name;
  unsigned long int max;
  unsigned long int min;
  size_t size;
} gsl_rng_type;

typedef struct {
  const gsl_rng_type *type;
  void *state;
} gsl_rng;

extern const gsl_rng_type *gsl_rng_mt19937;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long int seed);
unsigned long int gsl_rng_max(const gsl_rng *r);
unsigned long int gsl_rng_min(const gsl_rng *r);
unsigned long int gsl_rng_get(const gsl_rng *r);
unsigned long int gsl_rng_uniform_int(const gsl_rng *r, unsigned long int n);
void gsl_rng_free(gsl_rng *r);
int gsl_rng_fwrite(FILE *stream, const gsl_rng *r);
int gsl_rng_fread(FILE *stream, gsl_rng *r);

/* Replay support (not part of GSL). */
void hsmc_shim_script_raw(const unsigned long *vals, size_t n);
void hsmc_shim_script_int(const int *vals, size_t n);
void hsmc_shim_script_off(void);
size_t hsmc_shim_script_left_raw(void);
size_t hsmc_shim_script_left_int(void);

#endif
