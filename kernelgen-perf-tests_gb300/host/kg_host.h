/*
 * kg_host.h -- host-side helpers of the b200 target programs: the reference
 * main()'s input draws, coefficient lines and checksums, and timing.
 */
#ifndef KG_HOST_H
#define KG_HOST_H

#include <stddef.h>
#include <stdint.h>
#include <time.h>

#include "kg_b200.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Input variants. */
enum {
	KGH_INIT_REFERENCE = 0,    /* the reference main()'s rand() draws                 */
	KGH_INIT_BERNOULLI = 1,    /* gameoflife: 0/1 cells, P(1) = 0.3                   */
	KGH_INIT_UNIT_OFFSETS = 2, /* tricubic(2): offsets a, b, c uniform in [0,1)       */
	KGH_INIT_PULSE = 3         /* wave13pt/uxx1 precision sweep: Gaussian pulse
	                              (sigma 16 cells) + 1e-3 uniform noise, stable
	                              coefficients (see kg_host.c)                         */
};

/* glibc rand() as a per-object generator: after kgh_rng_seed(g, s) the
 * values of kgh_rng_next(g) equal those of rand() after srand(s).  glibc's
 * TYPE_3 additive feedback generator: r[0] = s, r[i] = 16807 r[i-1] mod
 * (2^31 - 1) for i < 31, r[i] = r[i-31] for i < 34, then
 * r[i] = r[i-3] + r[i-31] (mod 2^32), the first 310 discarded, output
 * r[i] >> 1.  Separate objects make independent streams for threads. */
typedef struct { uint32_t ring[34]; int k; } kgh_rng;
void kgh_rng_seed(kgh_rng* g, unsigned seed);
int kgh_rng_next(kgh_rng* g);

/* Test id of a suite directory name ("laplacian" ...), -1 if unknown. */
int kgh_test_id(const char* name);
const char* kgh_test_name(int test);

/* Seeds a kgh_rng with `seed` (1 is the reference's unseeded rand() state) and fills
 * coef[] and the arrays arrs[q] (nx*ny*ns doubles each, in kg_problem.arr
 * order) the way the reference main() draws them. */
void kgh_init(int test, int nx, int ny, int ns, int variant, unsigned seed,
	double* coef, double* const* arrs);

/* The reference's "initial mean": per index the arrays added left to right,
 * accumulated serially, / n / narr. */
double kgh_initial_mean(int test, size_t n, double* const* arrs);

/* Prints the coefficient line(s) the reference prints (none for tricubic,
 * tricubic2 and gameoflife). */
void kgh_print_coefs(int test, const double* coef);

/* timing.h equivalents (laplacian/timing.c:16-42), CLOCK_REALTIME. */
void kgh_get_time(struct timespec* t);
double kgh_time_diff(const struct timespec* a, const struct timespec* b);

#ifdef __cplusplus
}
#endif

#endif
