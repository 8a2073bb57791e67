/*
 * kg_oracle.c -- CPU restatement of the kernelgen-perf-tests stencil sweeps.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle; see kg_oracle.h).  Built twice by
 * oracle/Makefile: strict (-O2 -ffp-contract=off: the bitwise oracle) and
 * with the suite's fast-math flags plus OpenMP (the timed CPU baseline).
 *
 * Layout everywhere: x fastest, index ix + nx*iy + nx*ny*is
 * (laplacian/laplacian.c:30).  Outer loops carry an OpenMP pragma; splitting
 * the k (or j) loop over threads does not change any point's arithmetic.
 */
#include "kg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IX(i, j, k) ((size_t)(i) + (size_t)nx * ((size_t)(j) + (size_t)ny * (size_t)(k)))
#define IX2(i, j) ((size_t)(i) + (size_t)nx * (size_t)(j))

/* laplacian/laplacian.c:81-97 -- 7-point, interior [1,n-2]^3. */
void or_laplacian(int nx, int ny, int ns, double alpha, double beta,
	const double* w0, double* w1)
{
	#pragma omp parallel for schedule(static)
	for (int k = 1; k < ns - 1; k++)
		for (int j = 1; j < ny - 1; j++)
			for (int i = 1; i < nx - 1; i++)
				w1[IX(i, j, k)] = alpha * w0[IX(i, j, k)] + beta * (
					w0[IX(i + 1, j, k)] + w0[IX(i - 1, j, k)] +
					w0[IX(i, j + 1, k)] + w0[IX(i, j - 1, k)] +
					w0[IX(i, j, k + 1)] + w0[IX(i, j, k - 1)]);
}

/* divergence/divergence.c:84-97 -- u is the output, [1,n-2]^3. */
void or_divergence(int nx, int ny, int ns, double alpha, double beta, double gamma,
	double* u, const double* ux, const double* uy, const double* uz)
{
	#pragma omp parallel for schedule(static)
	for (int k = 1; k < ns - 1; k++)
		for (int j = 1; j < ny - 1; j++)
			for (int i = 1; i < nx - 1; i++)
				u[IX(i, j, k)] =
					alpha * (ux[IX(i + 1, j, k)] - ux[IX(i - 1, j, k)]) +
					beta  * (uy[IX(i, j + 1, k)] - uy[IX(i, j - 1, k)]) +
					gamma * (uz[IX(i, j, k + 1)] - uz[IX(i, j, k - 1)]);
}

/* gradient/gradient.c:85-98 -- three outputs, [1,n-2]^3. */
void or_gradient(int nx, int ny, int ns, double alpha, double beta, double gamma,
	const double* u, double* ux, double* uy, double* uz)
{
	#pragma omp parallel for schedule(static)
	for (int k = 1; k < ns - 1; k++)
		for (int j = 1; j < ny - 1; j++)
			for (int i = 1; i < nx - 1; i++)
			{
				ux[IX(i, j, k)] = alpha * (u[IX(i + 1, j, k)] - u[IX(i - 1, j, k)]);
				uy[IX(i, j, k)] = beta  * (u[IX(i, j + 1, k)] - u[IX(i, j - 1, k)]);
				uz[IX(i, j, k)] = gamma * (u[IX(i, j, k + 1)] - u[IX(i, j, k - 1)]);
			}
}

/* uxx1/uxx1.c:70,83-106 -- dth = 1/nx, domain [2,n-2]^3 (note: up to n-2). */
void or_uxx1(int nx, int ny, int ns, double c1, double c2,
	const double* u0, double* u1, const double* d1,
	const double* xx, const double* xy, const double* xz)
{
	double dth = 1. / nx;
	#pragma omp parallel for schedule(static)
	for (int k = 2; k < ns - 1; k++)
		for (int j = 2; j < ny - 1; j++)
			for (int i = 2; i < nx - 1; i++)
			{
				double d = 0.25 * (
					d1[IX(i, j, k    )] + d1[IX(i, j - 1, k    )] +
					d1[IX(i, j, k - 1)] + d1[IX(i, j - 1, k - 1)]);
				u1[IX(i, j, k)] = u0[IX(i, j, k)] + (dth / d) * (
					c1 * (xx[IX(i,     j,     k    )] - xx[IX(i - 1, j,     k    )]) +
					c2 * (xx[IX(i + 1, j,     k    )] - xx[IX(i - 2, j,     k    )]) +
					c1 * (xy[IX(i,     j,     k    )] - xy[IX(i,     j - 1, k    )]) +
					c2 * (xy[IX(i,     j + 1, k    )] - xy[IX(i,     j - 2, k    )]) +
					c1 * (xz[IX(i,     j,     k    )] - xz[IX(i,     j,     k - 1)]) +
					c2 * (xz[IX(i,     j,     k + 1)] - xz[IX(i,     j,     k - 2)]));
			}
}

/* wave13pt/wave13pt.c:146-154,214,640-651 (plain branch) -- [2,n-3]^3. */
void or_wave13pt(int nx, int ny, int ns, double m0, double m1, double m2,
	const double* w0, const double* w1, double* w2)
{
	#pragma omp parallel for schedule(static)
	for (int k = 2; k < ns - 2; k++)
		for (int j = 2; j < ny - 2; j++)
			for (int i = 2; i < nx - 2; i++)
				w2[IX(i, j, k)] = m0 * w1[IX(i, j, k)] - w0[IX(i, j, k)] +
					m1 * (
						w1[IX(i + 1, j, k)] + w1[IX(i - 1, j, k)] +
						w1[IX(i, j + 1, k)] + w1[IX(i, j - 1, k)] +
						w1[IX(i, j, k + 1)] + w1[IX(i, j, k - 1)]) +
					m2 * (
						w1[IX(i + 2, j, k)] + w1[IX(i - 2, j, k)] +
						w1[IX(i, j + 2, k)] + w1[IX(i, j - 2, k)] +
						w1[IX(i, j, k + 2)] + w1[IX(i, j, k - 2)]);
}

/* Lagrange cubic weights of tricubic/tricubic.c:1041-1054 (double branch),
 * same association: ((c * (a-1)) * a) * (a+1) and so on. */
static inline void tricubic_weights(double a, double w[4])
{
	w[0] =  1.0 / 6.0 * a * (a + 1.0) * (a + 2.0);
	w[1] = -0.5 * (a - 1.0) * (a + 1.0) * (a + 2.0);
	w[2] =  0.5 * (a - 1.0) * a * (a + 2.0);
	w[3] = -1.0 / 6.0 * (a - 1.0) * a * (a + 1.0);
}

/* tricubic/tricubic.c:138-155,509,1013-1145 -- [1,n-3]^3; the 64 terms
 * wX_a*wY_b*wZ_c*u0 summed left to right, x fastest then y then z. */
void or_tricubic(int nx, int ny, int ns, const double* u0, double* u1,
	const double* a, const double* b, const double* c)
{
	#pragma omp parallel for schedule(static)
	for (int k = 1; k < ns - 2; k++)
		for (int j = 1; j < ny - 2; j++)
			for (int i = 1; i < nx - 2; i++)
			{
				size_t p = IX(i, j, k);
				double wa[4], wb[4], wc[4];
				tricubic_weights(a[p], wa);
				tricubic_weights(b[p], wb);
				tricubic_weights(c[p], wc);
				double s = 0.0;
				int first = 1;
				for (int kk = 0; kk < 4; kk++)
					for (int jj = 0; jj < 4; jj++)
						for (int ii = 0; ii < 4; ii++)
						{
							double t = wa[ii] * wb[jj] * wc[kk] *
								u0[IX(i + ii - 1, j + jj - 1, k + kk - 1)];
							/* t0 + t1 + ... : the first term is not added to 0 */
							if (first) { s = t; first = 0; }
							else s = s + t;
						}
				u1[p] = s;
			}
}

/* tricubic2/tricubic2.c:68-102 -- [2,n-3]^3; u1 starts at 0 and accumulates
 * wa[ii]*wb[jj]*wc[kk]*u0 over kk, jj, ii. */
void or_tricubic2(int nx, int ny, int ns, const double* u0, double* u1,
	const double* a, const double* b, const double* c)
{
	#pragma omp parallel for schedule(static)
	for (int k = 2; k < ns - 2; k++)
		for (int j = 2; j < ny - 2; j++)
			for (int i = 2; i < nx - 2; i++)
			{
				size_t p = IX(i, j, k);
				double wa[4], wb[4], wc[4];
				tricubic_weights(a[p], wa);
				tricubic_weights(b[p], wb);
				tricubic_weights(c[p], wc);
				u1[p] = 0;
				for (int kk = 0; kk < 4; kk++)
					for (int jj = 0; jj < 4; jj++)
						for (int ii = 0; ii < 4; ii++)
							u1[p] += wa[ii] * wb[jj] * wc[kk] *
								u0[IX(i + ii - 1, j + jj - 1, k + kk - 1)];
			}
}

/* jacobi/jacobi.F90:60-67 -- Fortran w(i,j) 1-based, column major, i,j in
 * [2,n-1]; here 0-based [1,n-2] with index i + nx*j.  PARITY UNPINNED: the
 * kernel is Fortran and no Fortran compiler exists in this environment, so
 * this restatement follows the source text (left-to-right within the
 * parentheses, as gfortran evaluates without -ffast-math) and the PATUS spec
 * jacobi/jacobi.stc:9-11, and is checked only against itself. */
void or_jacobi(int nx, int ny, double c0, double c1, double c2,
	const double* w0, double* w1)
{
	#pragma omp parallel for schedule(static)
	for (int j = 1; j < ny - 1; j++)
		for (int i = 1; i < nx - 1; i++)
			w1[IX2(i, j)] = c0 * w0[IX2(i, j)] +
				c1 * (w0[IX2(i - 1, j)] + w0[IX2(i, j - 1)] + w0[IX2(i + 1, j)] + w0[IX2(i, j + 1)]) +
				c2 * (w0[IX2(i - 1, j - 1)] + w0[IX2(i - 1, j + 1)] + w0[IX2(i + 1, j - 1)] + w0[IX2(i + 1, j + 1)]);
}

/* lapgsrb/lapgsrb.c:81-117 -- out-of-place 25-point sweep, [2,n-3]^3. */
void or_lapgsrb(int nx, int ny, int ns, double c0, double c1, double c2, double c3,
	const double* w0, double* w1)
{
	#pragma omp parallel for schedule(static)
	for (int k = 2; k < ns - 2; k++)
		for (int j = 2; j < ny - 2; j++)
			for (int i = 2; i < nx - 2; i++)
				w1[IX(i, j, k)] = c0 * w0[IX(i, j, k)] +
					c1 * (
					w0[IX(i + 1, j, k)] + w0[IX(i - 1, j, k)] +
					w0[IX(i, j + 1, k)] + w0[IX(i, j - 1, k)] +
					w0[IX(i, j, k + 1)] + w0[IX(i, j, k - 1)]) +
					c2 * (
					w0[IX(i + 1, j + 1, k)] + w0[IX(i + 1, j, k + 1)] + w0[IX(i + 1, j, k - 1)] + w0[IX(i + 1, j - 1, k)] +
					w0[IX(i, j + 1, k + 1)] + w0[IX(i, j + 1, k - 1)] + w0[IX(i, j - 1, k + 1)] + w0[IX(i, j - 1, k - 1)] +
					w0[IX(i - 1, j + 1, k)] + w0[IX(i - 1, j, k + 1)] + w0[IX(i - 1, j, k - 1)] + w0[IX(i - 1, j - 1, k)]) +
					c3 * (
					w0[IX(i + 2, j, k)] + w0[IX(i - 2, j, k)] +
					w0[IX(i, j + 2, k)] + w0[IX(i, j - 2, k)] +
					w0[IX(i, j, k + 2)] + w0[IX(i, j, k - 2)]);
}

/* gaussblur/gaussblur.c:65,76-92 -- 5x5 blur, f computed per call, [2,n-3]^2. */
void or_gaussblur(int nx, int ny, double s0, double s1, double s2,
	double s4, double s5, double s8, const double* w0, double* w1)
{
	double f = 1. / (s0 + 4 * (s1 + s2 + s4 + s8) + 8 * s5);
	#pragma omp parallel for schedule(static)
	for (int j = 2; j < ny - 2; j++)
		for (int i = 2; i < nx - 2; i++)
			w1[IX2(i, j)] = f * (
				s0 *  w0[IX2(i,     j    )] +
				s1 * (w0[IX2(i - 1, j    )] + w0[IX2(i + 1, j    )] + w0[IX2(i,     j - 1)] + w0[IX2(i,     j + 1)]) +
				s2 * (w0[IX2(i - 1, j - 1)] + w0[IX2(i + 1, j - 1)] + w0[IX2(i - 1, j + 1)] + w0[IX2(i + 1, j + 1)]) +
				s4 * (w0[IX2(i - 2, j    )] + w0[IX2(i + 2, j    )] + w0[IX2(i,     j - 2)] + w0[IX2(i,     j + 2)]) +
				s5 * (w0[IX2(i - 2, j - 1)] + w0[IX2(i - 1, j - 2)] + w0[IX2(i + 1, j - 2)] + w0[IX2(i + 2, j - 1)] +
				      w0[IX2(i - 2, j + 1)] + w0[IX2(i - 1, j + 2)] + w0[IX2(i + 1, j + 2)] + w0[IX2(i + 2, j + 1)]) +
				s8 * (w0[IX2(i - 2, j - 2)] + w0[IX2(i + 2, j - 2)] + w0[IX2(i - 2, j + 2)] + w0[IX2(i + 2, j + 2)]));
}

/* gameoflife/gameoflife.c:76-91 -- smooth Conway rule on real cells, [1,n-2]^2. */
void or_gameoflife(int nx, int ny, const double* u0, double* u1)
{
	#pragma omp parallel for schedule(static)
	for (int j = 1; j < ny - 1; j++)
		for (int i = 1; i < nx - 1; i++)
		{
			double C = 100000000000000000000.;
			double L =
				u0[IX2(i - 1, j - 1)] + u0[IX2(i, j - 1)] + u0[IX2(i + 1, j - 1)] +
				u0[IX2(i - 1, j    )]                     + u0[IX2(i + 1, j    )] +
				u0[IX2(i - 1, j + 1)] + u0[IX2(i, j + 1)] + u0[IX2(i + 1, j + 1)];
			u1[IX2(i, j)] = 1. / (1. + (u0[IX2(i, j)] + L - 3.) * (L - 3.) * C);
		}
}

void or_conway_u8(int nx, int ny, const uint8_t* u0, uint8_t* u1)
{
	#pragma omp parallel for schedule(static)
	for (int j = 1; j < ny - 1; j++)
		for (int i = 1; i < nx - 1; i++)
		{
			int L = u0[IX2(i - 1, j - 1)] + u0[IX2(i, j - 1)] + u0[IX2(i + 1, j - 1)] +
				u0[IX2(i - 1, j)] + u0[IX2(i + 1, j)] +
				u0[IX2(i - 1, j + 1)] + u0[IX2(i, j + 1)] + u0[IX2(i + 1, j + 1)];
			int u = u0[IX2(i, j)];
			/* (u + L - 3) * (L - 3) == 0  <=>  alive in the reference rule */
			u1[IX2(i, j)] = (uint8_t)((u + L - 3) * (L - 3) == 0);
		}
}

/* ---- test programs ------------------------------------------------------ */

static const int k_narr[OR_NTESTS] = { 2, 4, 4, 6, 3, 5, 5, 2, 2, 2, 2 };
static const int k_ncoef[OR_NTESTS] = { 2, 3, 3, 2, 3, 0, 0, 3, 4, 6, 0 };

/* Threads of the OpenMP loops (the suite's gcc target itself is serial). */
void or_set_threads(int n)
{
#ifdef _OPENMP
	if (n > 0) omp_set_num_threads(n);
#else
	(void)n;
#endif
}

int or_narrays(int test) { return (test >= 0 && test < OR_NTESTS) ? k_narr[test] : -1; }
int or_ncoefs(int test) { return (test >= 0 && test < OR_NTESTS) ? k_ncoef[test] : -1; }
int or_is2d(int test) { return test == OR_JACOBI || test == OR_GAUSSBLUR || test == OR_GAMEOFLIFE; }

/* laplacian/laplacian.c:112 real_rand() with real = double. */
static double real_rand(void)
{
	return ((double)(rand() / (double)RAND_MAX) - 0.5) * 2;
}

void or_init(or_case* c, int variant, unsigned seed)
{
	const size_t n = (size_t)c->nx * c->ny * c->ns;
	c->narr = k_narr[c->test];
	c->ncoef = k_ncoef[c->test];
	for (int q = 0; q < 6; q++) { c->order[q] = q; c->coef[q] = 0; }
	srand(seed);

	/* Coefficient draws, in the reference's order. */
	switch (c->test)
	{
	case OR_LAPLACIAN:   /* laplacian/laplacian.c:141-142 */
		c->coef[0] = real_rand(); c->coef[1] = real_rand(); break;
	case OR_DIVERGENCE:  /* divergence/divergence.c:140-142 */
	case OR_GRADIENT:    /* gradient/gradient.c:141-143 */
		c->coef[0] = real_rand(); c->coef[1] = real_rand(); c->coef[2] = real_rand(); break;
	case OR_UXX1:        /* uxx1/uxx1.c:149-150 */
		c->coef[0] = real_rand(); c->coef[1] = real_rand(); break;
	case OR_WAVE13PT:    /* wave13pt/wave13pt.c:729-731 */
		c->coef[0] = real_rand(); c->coef[1] = real_rand() / 6.; c->coef[2] = real_rand() / 6.; break;
	case OR_JACOBI:      /* jacobi/main.c:90-92 */
		c->coef[0] = real_rand(); c->coef[1] = real_rand() / 4.; c->coef[2] = real_rand() / 4.; break;
	case OR_LAPGSRB:     /* lapgsrb/lapgsrb.c:161-164 */
		c->coef[0] = real_rand(); c->coef[1] = real_rand() / 6.;
		c->coef[2] = real_rand() / 12.; c->coef[3] = real_rand() / 6.; break;
	case OR_GAUSSBLUR:   /* gaussblur/gaussblur.c:134-139 */
		for (int q = 0; q < 6; q++) c->coef[q] = real_rand();
		break;
	default: break;      /* tricubic, tricubic2, gameoflife draw none */
	}

	/* Array draws, interleaved per index (laplacian/laplacian.c:158-164 and
	 * the per-test equivalents listed in k_narr order). */
	const int na = c->narr;
	for (size_t i = 0; i < n; i++)
	{
		for (int q = 0; q < na; q++)
		{
			double v;
			if (variant == OR_INIT_BERNOULLI)
				v = (rand() < 0.3 * ((double)RAND_MAX + 1.0)) ? 1.0 : 0.0;
			else if (variant == OR_INIT_UNIT_OFFSETS && q >= 2 &&
				(c->test == OR_TRICUBIC || c->test == OR_TRICUBIC2))
				v = rand() / ((double)RAND_MAX + 1.0);
			else
				v = real_rand();
			c->arr[q][i] = v;
		}
	}
}

void or_init_bernoulli_u8(int n, uint8_t* u0, uint8_t* u1, double p, unsigned seed)
{
	srand(seed);
	const double thr = p * ((double)RAND_MAX + 1.0);
	for (int i = 0; i < n; i++)
	{
		u0[i] = (uint8_t)(rand() < thr);
		u1[i] = (uint8_t)(rand() < thr);
	}
}

void or_sweep(or_case* c)
{
	const int nx = c->nx, ny = c->ny, ns = c->ns;
	double* const* a = c->arr;
	const double* k = c->coef;
	switch (c->test)
	{
	case OR_LAPLACIAN:  or_laplacian(nx, ny, ns, k[0], k[1], a[0], a[1]); break;
	case OR_DIVERGENCE: or_divergence(nx, ny, ns, k[0], k[1], k[2], a[0], a[1], a[2], a[3]); break;
	case OR_GRADIENT:   or_gradient(nx, ny, ns, k[0], k[1], k[2], a[0], a[1], a[2], a[3]); break;
	case OR_UXX1:       or_uxx1(nx, ny, ns, k[0], k[1], a[0], a[1], a[2], a[3], a[4], a[5]); break;
	case OR_WAVE13PT:   or_wave13pt(nx, ny, ns, k[0], k[1], k[2], a[0], a[1], a[2]); break;
	case OR_TRICUBIC:   or_tricubic(nx, ny, ns, a[0], a[1], a[2], a[3], a[4]); break;
	case OR_TRICUBIC2:  or_tricubic2(nx, ny, ns, a[0], a[1], a[2], a[3], a[4]); break;
	case OR_JACOBI:     or_jacobi(nx, ny * ns, k[0], k[1], k[2], a[0], a[1]); break;
	case OR_LAPGSRB:    or_lapgsrb(nx, ny, ns, k[0], k[1], k[2], k[3], a[0], a[1]); break;
	case OR_GAUSSBLUR:  or_gaussblur(nx, ny * ns, k[0], k[1], k[2], k[3], k[4], k[5], a[0], a[1]); break;
	case OR_GAMEOFLIFE: or_gameoflife(nx, ny * ns, a[0], a[1]); break;
	default: break;
	}
}

static void swap_slots(or_case* c, int p, int q)
{
	double* t = c->arr[p]; c->arr[p] = c->arr[q]; c->arr[q] = t;
	int o = c->order[p]; c->order[p] = c->order[q]; c->order[q] = o;
}

/* Loops of laplacian/laplacian.c:287-301 (2-buffer swap), wave13pt/wave13pt.c:
 * 907-921 (3-level rotation), divergence/divergence.c:297-309 and
 * gradient/gradient.c:303-315 (no swap). */
void or_run(or_case* c, int nt)
{
	for (int it = 0; it < nt; it++)
	{
		or_sweep(c);
		switch (c->test)
		{
		case OR_DIVERGENCE: case OR_GRADIENT: break;
		case OR_WAVE13PT:
			/* w0p = w1p; w1p = w2p; w2p = old w0p */
			swap_slots(c, 0, 1); swap_slots(c, 1, 2); break;
		default:
			swap_slots(c, 0, 1); break;
		}
	}
}

void or_rbsor_sweep(int nx, int ny, int ns, double omega, double* u, const double* f)
{
	for (int color = 0; color < 2; color++)
		for (int k = 1; k < ns - 1; k++)
			for (int j = 1; j < ny - 1; j++)
				for (int i = 1; i < nx - 1; i++)
				{
					if (((i + j + k) & 1) != color) continue;
					const size_t c = IX(i, j, k);
					const double s = u[c - 1] + u[c + 1] + u[c - nx] + u[c + nx] +
						u[c - (size_t)nx * ny] + u[c + (size_t)nx * ny];
					u[c] = u[c] + omega * ((s + f[c]) * (1.0 / 6.0) - u[c]);
				}
}

double or_residual_norm(int nx, int ny, int ns, const double* u, const double* f)
{
	double acc = 0.0;
	for (int k = 1; k < ns - 1; k++)
		for (int j = 1; j < ny - 1; j++)
			for (int i = 1; i < nx - 1; i++)
			{
				const size_t c = IX(i, j, k);
				const double au = 6.0 * u[c] - (u[c - 1] + u[c + 1] + u[c - nx] + u[c + nx] +
					u[c - (size_t)nx * ny] + u[c + (size_t)nx * ny]);
				const double r = f[c] - au;
				acc += r * r;
			}
	return sqrt(acc);
}

double or_sum(const double* x, size_t n)
{
	double s = 0.0;
	for (size_t i = 0; i < n; i++) s += x[i];
	return s;
}

double or_initial_mean(const or_case* c)
{
	const size_t n = (size_t)c->nx * c->ny * c->ns;
	double mean = 0.0;
	for (size_t i = 0; i < n; i++)
	{
		double t = c->arr[0][i];
		for (int q = 1; q < c->narr; q++) t = t + c->arr[q][i];
		mean += t;
	}
	return mean / n / c->narr;
}

int or_final_slot(const or_case* c)
{
	switch (c->test)
	{
	case OR_DIVERGENCE: return 0;   /* divergence/divergence.c:378-381: u */
	case OR_GRADIENT:   return -1;  /* gradient/gradient.c:388-391: (ux+uy+uz)/3 */
	default:            return 1;   /* w[idxs[1]] (laplacian/laplacian.c:307-313,374-377) */
	}
}

double or_final_mean(const or_case* c)
{
	const size_t n = (size_t)c->nx * c->ny * c->ns;
	double mean = 0.0;
	if (c->test == OR_GRADIENT)
	{
		for (size_t i = 0; i < n; i++) mean += c->arr[1][i] + c->arr[2][i] + c->arr[3][i];
		return mean / n / 3;
	}
	const double* w = c->arr[or_final_slot(c)];
	for (size_t i = 0; i < n; i++) mean += w[i];
	return mean / n;
}
