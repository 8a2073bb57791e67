/*
 * kg_oracle_extra.c -- CPU restatement of the suite's tests that are not
 * stencil sweeps: vecadd, matvec, matmul, sincos, whispering.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle), like kg_oracle.c.  Each kernel
 * follows the reference loop and expression in order; each *_program
 * reproduces the reference main(): rand() draws in its order (the reference
 * never seeds: srand(1)), the time loop with its pointer rotation, and the
 * printed means with its accumulation order.  Citations are file:line inside
 * the reference project.  Loops whose outputs are independent run as OpenMP
 * loops (each output is computed exactly as in the serial loop); whispering's
 * in-place loop stays serial.
 *
 * Pins: vecadd, matvec and whispering are C in the reference and are checked
 * against its own sources compiled unmodified (tests/golden/
 * reference_extra.json).  matmul and sincos are Fortran kernels
 * (matmul/matmul.F90, sincos/sincos.F90) and no Fortran compiler exists here:
 * their restatements are PARITY UNPINNED (their README.md rows are FAIL).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "kg_oracle.h"

/* laplacian/laplacian.c:112 (the same macro in every test's source). */
static double real_rand(void)
{
	return ((double)(rand() / (double)RAND_MAX) - 0.5) * 2;
}

/* ---- kernels ---------------------------------------------------------- */

/* vecadd/vecadd.c:38-84 */
void or_vecadd(size_t n, const double* w0, const double* w1, double* w2)
{
	#pragma omp parallel for
	for (size_t i = 0; i < n; i++) w2[i] = w0[i] + w1[i];
}

/* matvec/matvec.c:37-71: y[j] = 0; y[j] += A[i + nx*j] * x[i] */
void or_matvec(int nx, int ny, const double* A, const double* x, double* y)
{
	#pragma omp parallel for
	for (int j = 0; j < ny; j++) {
		double s = 0;
		for (int i = 0; i < nx; i++) s += A[i + (size_t)nx * j] * x[i];
		y[j] = s;
	}
}

/* matmul/matmul.F90:56-68, column-major: C(i,j) = C(i,j) + A(i,k) * B(k,j). */
void or_matmul(int nx, int ny, int ns, const double* A, const double* B, double* C)
{
	#pragma omp parallel for
	for (int j = 0; j < ns; j++)
		for (int i = 0; i < nx; i++) {
			double c = C[i + (size_t)nx * j];
			for (int k = 0; k < ny; k++) c = c + A[i + (size_t)nx * k] * B[k + (size_t)ny * j];
			C[i + (size_t)nx * j] = c;
		}
}

/* sincos/sincos.F90:60-72 */
void or_sincos(size_t n, const double* x, const double* y, double* xy)
{
	#pragma omp parallel for
	for (size_t i = 0; i < n; i++) xy[i] = sin(x[i]) + cos(y[i]);
}

/* whispering/whispering.c:87-108, in the reference's loop order (e is
 * updated in place; e component c of (i, j) at e[i + nx*j + nx*ny*c]). */
void or_whispering(int nx, int ny, double mu, double epsilon, double* e, const double* h0, double* h1,
	const double* u_em0, double* u_em1, const double* ca, const double* cb, const double* da, const double* db)
{
	const size_t p = (size_t)nx * ny;
#define A2(a, i, j) ((a)[(i) + (size_t)nx * (j)])
	for (int j = 1; j < ny - 1; j++)
		for (int i = 1; i < nx - 1; i++) {
			double e0 = A2(ca, i, j) * A2(e, i, j) + A2(cb, i, j) * (A2(h0, i, j + 1) - A2(h0, i, j));
			double e1 = A2(ca, i, j) * A2(e + p, i, j) - A2(cb, i, j) * (A2(h0, i + 1, j) - A2(h0, i, j));
			double ey = A2(ca, i, j - 1) * A2(e, i, j - 1) + A2(cb, i, j - 1) * (A2(h0, i, j) - A2(h0, i, j - 1));
			double ex = A2(ca, i - 1, j) * A2(e + p, i - 1, j) - A2(cb, i - 1, j) * (A2(h0, i, j) - A2(h0, i - 1, j));
			A2(e, i, j) = e0;
			A2(e + p, i, j) = e1;
			double h = A2(da, i, j) * A2(h0, i, j) + A2(db, i, j) * (e0 - ey + ex - e1);
			A2(h1, i, j) = h;
			A2(u_em1, i, j) = A2(u_em0, i, j) + 0.5 * (h * h / mu + epsilon * (e0 * e0 + e1 * e1));
		}
#undef A2
}

/* ---- whole programs ------------------------------------------------------ */

/* vecadd/vecadd.c:137-145 draws (per index w0, w1, w2), :276-279 loop with
 * the three-level rotation, :365-369 final mean over w1. */
void or_vecadd_program(int nx, int ny, int ns, int nt, double** w, double* imean, double* fmean)
{
	const size_t n = (size_t)nx * ny * ns;
	srand(1);
	double mean = 0.0;
	for (size_t i = 0; i < n; i++) {
		w[0][i] = real_rand();
		w[1][i] = real_rand();
		w[2][i] = real_rand();
		mean += w[0][i] + w[1][i] + w[2][i];
	}
	*imean = mean / n / 3;
	for (int it = 0; it < nt; it++) {
		or_vecadd(n, w[0], w[1], w[2]);
		double* t = w[0]; w[0] = w[1]; w[1] = w[2]; w[2] = t;
	}
	mean = 0.0;
	for (size_t i = 0; i < n; i++) mean += w[1][i];
	*fmean = mean / n;
}

/* matvec/matvec.c:120-140 draws (A, then x, then y), nt identical products,
 * :337-340 final mean of y. */
void or_matvec_program(int nx, int ny, int nt, double* A, double* x, double* y, double* imean, double* fmean)
{
	srand(1);
	double amean = 0.0, xmean = 0.0, ymean = 0.0;
	for (size_t i = 0; i < (size_t)nx * ny; i++) { A[i] = real_rand(); amean += A[i]; }
	for (int i = 0; i < nx; i++) { x[i] = real_rand(); xmean += x[i]; }
	for (int i = 0; i < ny; i++) { y[i] = real_rand(); ymean += y[i]; }
	*imean = amean / ((double)nx * ny) + xmean / nx + ymean / ny;
	for (int it = 0; it < nt; it++) or_matvec(nx, ny, A, x, y);
	ymean = 0.0;
	for (int i = 0; i < ny; i++) ymean += y[i];
	*fmean = ymean / ny;
}

/* matmul/main.c:98-110 draws (A, then B); C starts at zero (the reference
 * leaves it unset; freshly mapped memory is zero); nt accumulations;
 * :311-314 final mean of C. */
void or_matmul_program(int nx, int ny, int ns, int nt, double* A, double* B, double* C, double* imean, double* fmean)
{
	const size_t na = (size_t)nx * ny, nb = (size_t)ny * ns, nc = (size_t)nx * ns;
	srand(1);
	double ma = 0.0, mb = 0.0;
	for (size_t i = 0; i < na; i++) { A[i] = real_rand(); ma += A[i]; }
	for (size_t i = 0; i < nb; i++) { B[i] = real_rand(); mb += B[i]; }
	*imean = ma / na + mb / nb;
	memset(C, 0, nc * sizeof(double));
	for (int it = 0; it < nt; it++) or_matmul(nx, ny, ns, A, B, C);
	double mc = 0.0;
	for (size_t i = 0; i < nc; i++) mc += C[i];
	*fmean = mc / nc;
}

/* sincos/main.c:99-107 draws (per index x, y, xy), :311-316 final mean. */
void or_sincos_program(int nx, int ny, int ns, int nt, double* x, double* y, double* xy, double* imean, double* fmean)
{
	const size_t n = (size_t)nx * ny * ns;
	srand(1);
	double mean = 0.0;
	for (size_t i = 0; i < n; i++) {
		x[i] = real_rand();
		y[i] = real_rand();
		xy[i] = real_rand();
		mean += x[i] + y[i] + xy[i];
	}
	*imean = mean / n / 3;
	for (int it = 0; it < nt; it++) or_sincos(n, x, y, xy);
	mean = 0.0;
	for (size_t i = 0; i < n; i++) mean += xy[i];
	*fmean = mean / n;
}

/* whispering/whispering.c:148-190 draws (mu, epsilon, then per index e[2i],
 * e[2i+1], h0, h1, u_em0, u_em1, ca, cb, da, db), :356-371 loop swapping h
 * and u_em, :471-476 final mean.  a[] = e (2 n), h0, h1, u_em0, u_em1, ca,
 * cb, da, db; on return a[1..4] hold h0, h1, u_em0, u_em1 in their final
 * roles. */
void or_whispering_program(int nx, int ny, int nt, double* coef, double** a, double* imean, double* fmean)
{
	const size_t n = (size_t)nx * ny;
	srand(1);
	coef[0] = real_rand();
	coef[1] = real_rand();
	double mean = 0.0;
	for (size_t i = 0; i < n; i++) {
		a[0][2 * i] = real_rand();
		a[0][2 * i + 1] = real_rand();
		for (int q = 1; q < 9; q++) a[q][i] = real_rand();
		mean += a[0][2 * i] + a[0][2 * i + 1] + a[1][i] + a[2][i] + a[3][i] + a[4][i] +
			a[5][i] + a[6][i] + a[7][i] + a[8][i];
	}
	*imean = mean / n / 12;
	for (int it = 0; it < nt; it++) {
		or_whispering(nx, ny, coef[0], coef[1], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]);
		double* t = a[1]; a[1] = a[2]; a[2] = t;
		t = a[3]; a[3] = a[4]; a[4] = t;
	}
	mean = 0.0;
	for (size_t i = 0; i < n; i++) mean += a[0][2 * i] + a[0][2 * i + 1] + a[2][i] + a[4][i];
	*fmean = mean / n / 4;
}
