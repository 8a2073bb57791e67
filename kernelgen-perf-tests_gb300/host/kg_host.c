/*
 * kg_host.c -- host-side helpers of the b200 target programs.
 *
 * Inputs come from kgh_rng, a re-implementation of glibc's rand(), so that
 * independent generators can fill several test programs in parallel.
 *
 * Compiled with -ffp-contract=off -fno-fast-math: the input values must be
 * the IEEE evaluation of the reference's real_rand() expression
 * (laplacian/laplacian.c:112), so that the arrays handed to the GPU equal
 * the ones a strict build of the reference computes, bit for bit.
 */
#include "kg_host.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static const char* k_names[KG_NSTENCILS] = {
	"laplacian", "divergence", "gradient", "uxx1", "wave13pt", "tricubic",
	"tricubic2", "jacobi", "lapgsrb", "gaussblur", "gameoflife"
};

int kgh_test_id(const char* name)
{
	for (int t = 0; t < KG_NSTENCILS; t++)
		if (name && strcmp(name, k_names[t]) == 0) return t;
	return -1;
}

const char* kgh_test_name(int test)
{
	return (test >= 0 && test < KG_NSTENCILS) ? k_names[test] : "?";
}

void kgh_rng_seed(kgh_rng* g, unsigned seed)
{
	int32_t r0 = (int32_t)(seed ? seed : 1u);
	g->ring[0] = (uint32_t)r0;
	for (int i = 1; i < 31; i++) {
		/* 16807 * r mod (2^31 - 1) without overflow (Schrage) */
		const int32_t hi = r0 / 127773, lo = r0 % 127773;
		int32_t w = 16807 * lo - 2836 * hi;
		if (w < 0) w += 2147483647;
		g->ring[i] = (uint32_t)w;
		r0 = w;
	}
	for (int i = 31; i < 34; i++) g->ring[i] = g->ring[i - 31];
	g->k = 0;  /* next index 34 maps to ring slot 0 */
	for (int i = 0; i < 310; i++) kgh_rng_next(g);
}

int kgh_rng_next(kgh_rng* g)
{
	/* r[i] = r[i-31] + r[i-3]; with i = 34 + m, slot (i mod 34) = k */
	const int k = g->k;
	const uint32_t v = g->ring[(k + 3) % 34] + g->ring[(k + 31) % 34];
	g->ring[k] = v;
	g->k = (k + 1) % 34;
	return (int)(v >> 1);
}

#define KGH_RAND_MAX 2147483647

/* laplacian/laplacian.c:112 real_rand() with real = double. */
static double real_rand(kgh_rng* g)
{
	return ((double)(kgh_rng_next(g) / (double)KGH_RAND_MAX) - 0.5) * 2;
}

/* Uniform [0,1). */
static double unit_rand(kgh_rng* g)
{
	return kgh_rng_next(g) / ((double)KGH_RAND_MAX + 1.0);
}

/* Precision-sweep init: a Gaussian pulse of sigma = 16 cells centred in the
 * box plus 1e-3 * uniform[-1,1) noise, for every array of the test; uxx1's
 * density d1 becomes 1 + pulse (bounded away from 0). */
static double pulse(int nx, int ny, int ns, size_t idx)
{
	const size_t i = idx % (size_t)nx, j = (idx / (size_t)nx) % (size_t)ny, k = idx / ((size_t)nx * ny);
	const double x = (double)i - 0.5 * (nx - 1), y = (double)j - 0.5 * (ny - 1), z = (double)k - 0.5 * (ns - 1);
	const double s = 16.0;
	return exp(-(x * x + y * y + z * z) / (2.0 * s * s));
}

void kgh_init(int test, int nx, int ny, int ns, int variant, unsigned seed,
	double* coef, double* const* arrs)
{
	const size_t n = (size_t)nx * ny * ns;
	const int narr = kg_stencil_narrays(test);
	for (int q = 0; q < 6; q++) coef[q] = 0.0;
	kgh_rng gen;
	kgh_rng* g = &gen;
	kgh_rng_seed(g, seed);

	if (variant == KGH_INIT_PULSE) {
		/* Stable coefficients (project-defined; the reference's random ones
		 * are not a stable time step).  wave13pt: the 4th-order leapfrog
		 * w2 = 2 w1 - w0 + C^2 (-15/2 w1 + 4/3 sum_r1 - 1/12 sum_r2), Courant
		 * number C = 0.4.  uxx1: c1 = 9/8, c2 = -1/24 (4th-order staggered). */
		if (test == KG_WAVE13PT) {
			const double c2 = 0.4 * 0.4;
			coef[0] = 2.0 - c2 * 7.5;
			coef[1] = c2 * (4.0 / 3.0);
			coef[2] = -c2 / 12.0;
		} else if (test == KG_UXX1) {
			coef[0] = 9.0 / 8.0;
			coef[1] = -1.0 / 24.0;
		}
		/* The noise of plane k comes from its own generator, seeded with
		 * seed + k + 1, so planes fill in parallel and the result does not
		 * depend on the thread count. */
		#pragma omp parallel for schedule(dynamic, 1)
		for (int k = 0; k < ns; k++) {
			kgh_rng pg;
			kgh_rng_seed(&pg, seed + (unsigned)k + 1u);
			const size_t i0 = (size_t)k * nx * ny, i1 = i0 + (size_t)nx * ny;
			for (size_t i = i0; i < i1; i++) {
				const double gp = pulse(nx, ny, ns, i);
				for (int q = 0; q < narr; q++) {
					double v = gp + 1e-3 * real_rand(&pg);
					if (test == KG_UXX1 && q == 2) v = 1.0 + v;
					arrs[q][i] = v;
				}
			}
		}
		return;
	}

	switch (test) {
	case KG_LAPLACIAN:   /* laplacian/laplacian.c:141-142 */
	case KG_UXX1:        /* uxx1/uxx1.c:149-150 */
		coef[0] = real_rand(g); coef[1] = real_rand(g); break;
	case KG_DIVERGENCE:  /* divergence/divergence.c:140-142 */
	case KG_GRADIENT:    /* gradient/gradient.c:141-143 */
		coef[0] = real_rand(g); coef[1] = real_rand(g); coef[2] = real_rand(g); break;
	case KG_WAVE13PT:    /* wave13pt/wave13pt.c:729-731 */
		coef[0] = real_rand(g); coef[1] = real_rand(g) / 6.; coef[2] = real_rand(g) / 6.; break;
	case KG_JACOBI:      /* jacobi/main.c:90-92 */
		coef[0] = real_rand(g); coef[1] = real_rand(g) / 4.; coef[2] = real_rand(g) / 4.; break;
	case KG_LAPGSRB:     /* lapgsrb/lapgsrb.c:161-164 */
		coef[0] = real_rand(g); coef[1] = real_rand(g) / 6.;
		coef[2] = real_rand(g) / 12.; coef[3] = real_rand(g) / 6.; break;
	case KG_GAUSSBLUR:   /* gaussblur/gaussblur.c:134-139 */
		for (int q = 0; q < 6; q++) coef[q] = real_rand(g);
		break;
	default: break;
	}

	/* Interleaved per index, arrays in allocation order
	 * (laplacian/laplacian.c:158-164 and its per-test equivalents). */
	const double thr = 0.3 * ((double)KGH_RAND_MAX + 1.0);
	const int offsets = (variant == KGH_INIT_UNIT_OFFSETS) &&
		(test == KG_TRICUBIC || test == KG_TRICUBIC2);
	for (size_t i = 0; i < n; i++) {
		for (int q = 0; q < narr; q++) {
			double v;
			if (variant == KGH_INIT_BERNOULLI) v = (kgh_rng_next(g) < thr) ? 1.0 : 0.0;
			else if (offsets && q >= 2) v = unit_rand(g);
			else v = real_rand(g);
			arrs[q][i] = v;
		}
	}
}

double kgh_initial_mean(int test, size_t n, double* const* arrs)
{
	const int narr = kg_stencil_narrays(test);
	double mean = 0.0;
	for (size_t i = 0; i < n; i++) {
		double t = arrs[0][i];
		for (int q = 1; q < narr; q++) t = t + arrs[q][i];
		mean += t;
	}
	return mean / n / narr;
}

void kgh_print_coefs(int test, const double* c)
{
	switch (test) {
	case KG_LAPLACIAN: printf("alpha = %f, beta = %f\n", c[0], c[1]); break;
	case KG_DIVERGENCE:
	case KG_GRADIENT: printf("alpha = %f, beta = %f, gamma = %f\n", c[0], c[1], c[2]); break;
	case KG_UXX1: printf("c1 = %f, c2 = %f\n", c[0], c[1]); break;
	case KG_WAVE13PT: printf("m0 = %f, m1 = %f, m2 = %f\n", c[0], c[1], c[2]); break;
	case KG_JACOBI: printf("c0 = %f, c1 = %f, c2 = %f\n", c[0], c[1], c[2]); break;
	case KG_LAPGSRB: printf("c0 = %f, c1 = %f, c2 = %f, c3 = %f\n", c[0], c[1], c[2], c[3]); break;
	case KG_GAUSSBLUR:
		printf("s0 = %f, s1 = %f, s2 = %f\n", c[0], c[1], c[2]);
		printf("s4 = %f, s5 = %f, s8 = %f\n", c[3], c[4], c[5]);
		break;
	default: break;
	}
}

void kgh_get_time(struct timespec* t)
{
	clock_gettime(CLOCK_REALTIME, t);
}

double kgh_time_diff(const struct timespec* a, const struct timespec* b)
{
	return (double)(b->tv_sec - a->tv_sec) + 1e-9 * (double)(b->tv_nsec - a->tv_nsec);
}
