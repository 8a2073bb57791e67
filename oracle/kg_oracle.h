/*
 * kg_oracle.h -- CPU restatement of the kernelgen-perf-tests stencil sweeps.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle: tests, the smoke
 * check and the CPU-baseline leg of bench.py call it; the product (the
 * sm_103a library and the b200 host drivers) never links or calls it.
 *
 * Every sweep follows the reference source expression term by term, in the
 * same association order, so that a build with -ffp-contract=off reproduces
 * an IEEE double evaluation of the reference bit for bit.  Citations are
 * file:line inside the reference project.
 *
 * Parity pins: the restatement is checked against (1) array hashes and
 * printed checksum lines produced by the reference's own C sources compiled
 * unmodified (tests/golden/, generated by tests/golden/make_golden.py), and
 * (2) the README.md:113-128 checksum table of the reference.  jacobi's kernel
 * is Fortran (jacobi/jacobi.F90) and no Fortran compiler exists here, so the
 * jacobi restatement is "parity unpinned" (see the jacobi section below).
 */
#ifndef KG_ORACLE_H
#define KG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Test ids; same numbering as kg_stencil in include/kg_b200.h. */
enum {
	OR_LAPLACIAN = 0, OR_DIVERGENCE = 1, OR_GRADIENT = 2, OR_UXX1 = 3,
	OR_WAVE13PT = 4, OR_TRICUBIC = 5, OR_TRICUBIC2 = 6, OR_JACOBI = 7,
	OR_LAPGSRB = 8, OR_GAUSSBLUR = 9, OR_GAMEOFLIFE = 10, OR_NTESTS = 11
};

/* Input variants of or_init(). */
enum {
	OR_INIT_REFERENCE = 0,   /* the reference main()'s rand() draws           */
	OR_INIT_BERNOULLI = 1,   /* gameoflife: 0/1 cells, P(1) = 0.3 (project)  */
	OR_INIT_UNIT_OFFSETS = 2 /* tricubic(2): offsets a,b,c in [0,1) (project)*/
};

/* One sweep of each reference kernel (FP64). */
void or_laplacian(int nx, int ny, int ns, double alpha, double beta,
	const double* w0, double* w1);
void or_divergence(int nx, int ny, int ns, double alpha, double beta, double gamma,
	double* u, const double* ux, const double* uy, const double* uz);
void or_gradient(int nx, int ny, int ns, double alpha, double beta, double gamma,
	const double* u, double* ux, double* uy, double* uz);
void or_uxx1(int nx, int ny, int ns, double c1, double c2,
	const double* u0, double* u1, const double* d1,
	const double* xx, const double* xy, const double* xz);
void or_wave13pt(int nx, int ny, int ns, double m0, double m1, double m2,
	const double* w0, const double* w1, double* w2);
void or_tricubic(int nx, int ny, int ns, const double* u0, double* u1,
	const double* a, const double* b, const double* c);
void or_tricubic2(int nx, int ny, int ns, const double* u0, double* u1,
	const double* a, const double* b, const double* c);
void or_jacobi(int nx, int ny, double c0, double c1, double c2,
	const double* w0, double* w1);
void or_lapgsrb(int nx, int ny, int ns, double c0, double c1, double c2, double c3,
	const double* w0, double* w1);
void or_gaussblur(int nx, int ny, double s0, double s1, double s2,
	double s4, double s5, double s8, const double* w0, double* w1);
void or_gameoflife(int nx, int ny, const double* u0, double* u1);

/* B3/S23 Conway on 0/1 byte cells over [1,n-2]^2, rims untouched.  This is the
 * integer form of or_gameoflife: fed 0/1 doubles, the reference rule yields
 * exactly 1.0 for a live cell and a value below 1e-19 for a dead one. */
void or_conway_u8(int nx, int ny, const uint8_t* u0, uint8_t* u1);

/* A whole test program: arrays in the order the reference main() allocates
 * them, coefficients in the order it draws them. */
typedef struct {
	int test;
	int nx, ny, ns;        /* 2D tests: ns = 1, ny = NY*NS as their makefiles pass */
	int narr;
	int ncoef;
	double coef[6];
	double* arr[6];        /* caller-owned, nx*ny*ns doubles each */
	int order[6];          /* arr[] slot currently holding original array q */
} or_case;

int or_narrays(int test);
int or_ncoefs(int test);
int or_is2d(int test);

/* Seed glibc rand() (the reference never seeds: srand(1) is its state) and
 * draw coefficients then arrays exactly as the reference main() does. */
void or_init(or_case* c, int variant, unsigned seed);
/* Bernoulli(p) 0/1 byte cells, both buffers interleaved per index. */
void or_init_bernoulli_u8(int n, uint8_t* u0, uint8_t* u1, double p, unsigned seed);

/* One sweep with the current array roles. */
void or_sweep(or_case* c);
/* Threads of the OpenMP loops of the fast build (no effect on the strict build). */
void or_set_threads(int n);
/* nt sweeps with the reference's pointer rotation after each sweep. */
void or_run(or_case* c, int nt);

/* Checksums as the reference prints them ("initial mean", "final mean"). */
double or_initial_mean(const or_case* c);
double or_final_mean(const or_case* c);
/* Index (into arr[]) of the buffer the final mean is taken over (ping-pong
 * tests: the input of the last sweep; wave13pt: the newest level). */
int or_final_slot(const or_case* c);

/* Red-black SOR for A u = f, A u = 6 u - (6 face neighbours), u = 0 on the
 * outer planes: one sweep = the red half ((i+j+k) even) then the black half,
 * u += omega * ((sum + f) / 6 - u).  Project-defined (PARITY UNPINNED: the
 * reference has no such solver; checked by its residual). */
void or_rbsor_sweep(int nx, int ny, int ns, double omega, double* u, const double* f);
/* ||f - A u||_2 over the interior. */
double or_residual_norm(int nx, int ny, int ns, const double* u, const double* f);

/* Plain FP64 serial sum of x[0..n). */
double or_sum(const double* x, size_t n);

/* ---- the suite's other tests (kg_oracle_extra.c) ------------------------ */
void or_vecadd(size_t n, const double* w0, const double* w1, double* w2);
void or_matvec(int nx, int ny, const double* A, const double* x, double* y);
void or_matmul(int nx, int ny, int ns, const double* A, const double* B, double* C);
void or_sincos(size_t n, const double* x, const double* y, double* xy);
void or_whispering(int nx, int ny, double mu, double epsilon, double* e, const double* h0, double* h1,
	const double* u_em0, double* u_em1, const double* ca, const double* cb, const double* da, const double* db);
/* Whole programs (reference draws, time loop, means); w / a permuted into
 * their final roles. */
void or_vecadd_program(int nx, int ny, int ns, int nt, double** w, double* imean, double* fmean);
void or_matvec_program(int nx, int ny, int nt, double* A, double* x, double* y, double* imean, double* fmean);
void or_matmul_program(int nx, int ny, int ns, int nt, double* A, double* B, double* C, double* imean, double* fmean);
void or_sincos_program(int nx, int ny, int ns, int nt, double* x, double* y, double* xy, double* imean, double* fmean);
void or_whispering_program(int nx, int ny, int nt, double* coef, double** a, double* imean, double* fmean);

#ifdef __cplusplus
}
#endif

#endif
