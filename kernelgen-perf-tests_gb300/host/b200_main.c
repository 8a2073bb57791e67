/*
 * b200_main.c -- the b200 target program of one suite test (KG_TEST_NAME).
 *
 * Same command line, input draws, phases and stdout lines as the reference
 * main() (laplacian/laplacian.c:114-385; 2D tests: gameoflife/gameoflife.c:
 * 107-372, jacobi/main.c:64-342), so the suite's `benchmark` harness parses it
 * (benchmark:137-282).  The sweeps run on the GPU through the kg_b200 C ABI.
 *
 * Knobs (environment, set by the target makefile from make variables):
 *   B200_PREC  fp64 (default; bitwise = IEEE reference) | fp64fma | fp64ff
 *              (FP64 storage, float-float arithmetic) | fp64mix (uxx1,
 *              wave13pt: FP64 state, FP32 increments) | fp32 | bf16 | fp16 |
 *              u8 (gameoflife on 0/1 byte cells)
 *   B200_INIT  reference (default) | bernoulli | unit | pulse
 *   B200_MODE  plain (default: one launch per sweep, timed) | graph (the
 *              nt-sweep loop replayed as one CUDA graph)
 *   B200_ENGINE auto (default) | direct | staged | tma | tmavec (kg_problem.engine)
 *   NO_TIMING, PROFILING_FNAME as in the reference.
 * With PROFILING_FNAME set it prints "<name> regcount = N" and, per sweep,
 * "<name> kernel time = t", the two lines the reference's launch interposer
 * prints (cuda_profiling.cu:236-249), with the same meaning: host wall time
 * from before the launch to after the device has synchronised.  As in the
 * reference's cuda branch (laplacian/laplacian.c:292-297) every plain-mode
 * sweep is followed by a device synchronisation.  The device time of each
 * sweep (CUDA events) follows as "<name> device time = t", a line the
 * harness does not parse.  In graph mode both are the replay's times / nt.
 */
#include <malloc.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cuda_runtime_api.h>

#include "kg_b200.h"
#include "kg_host.h"

#ifndef KG_TEST_NAME
#error "KG_TEST_NAME must name the suite test"
#endif

#define MEMALIGN 4096

static void die_kg(kg_status s, const char* what)
{
	fprintf(stderr, "Error \"%s: %s\" in %s\n", kg_status_string(s), kg_last_error(), what);
	exit(-1);
}

static void die_cuda(cudaError_t e, const char* what)
{
	fprintf(stderr, "Error \"%s\" in %s\n", cudaGetErrorString(e), what);
	exit(-1);
}

#define KG_CHECK(x) do { kg_status s_ = (x); if (s_ != KG_OK) die_kg(s_, #x); } while (0)
#define CU_CHECK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) die_cuda(e_, #x); } while (0)

static int parse_arg(const char* name, const char* arg)
{
	int v = atoi(arg);
	if (v < 0) {
		printf("Value for %s is invalid: %d\n", name, v);
		exit(1);
	}
	return v;
}

static kg_dtype parse_prec(const char* s)
{
	if (!s || !*s || !strcmp(s, "fp64")) return KG_F64;
	if (!strcmp(s, "fp64fma")) return KG_F64_FMA;
	if (!strcmp(s, "fp32")) return KG_F32;
	if (!strcmp(s, "bf16")) return KG_BF16;
	if (!strcmp(s, "fp16")) return KG_F16;
	if (!strcmp(s, "u8")) return KG_U8;
	if (!strcmp(s, "fp64ff")) return KG_F64_FF;
	if (!strcmp(s, "fp64mix")) return KG_F64_MIX;
	fprintf(stderr, "Unknown B200_PREC=%s\n", s);
	exit(1);
}

static int parse_engine(const char* s)
{
	if (!s || !*s || !strcmp(s, "auto")) return KG_ENGINE_AUTO;
	if (!strcmp(s, "direct")) return KG_ENGINE_DIRECT;
	if (!strcmp(s, "staged")) return KG_ENGINE_STAGED;
	if (!strcmp(s, "tma")) return KG_ENGINE_TMA;
	if (!strcmp(s, "tmavec")) return KG_ENGINE_TMA_VEC;
	fprintf(stderr, "Unknown B200_ENGINE=%s\n", s);
	exit(1);
}

static int parse_init(const char* s)
{
	if (!s || !*s || !strcmp(s, "reference")) return KGH_INIT_REFERENCE;
	if (!strcmp(s, "bernoulli")) return KGH_INIT_BERNOULLI;
	if (!strcmp(s, "unit")) return KGH_INIT_UNIT_OFFSETS;
	if (!strcmp(s, "pulse")) return KGH_INIT_PULSE;
	fprintf(stderr, "Unknown B200_INIT=%s\n", s);
	exit(1);
}

/* Pointer rotation after a sweep (laplacian/laplacian.c:299-300,
 * wave13pt/wave13pt.c:919; divergence and gradient keep their arrays). */
static void rotate(int test, void** a)
{
	void* t;
	if (test == KG_DIVERGENCE || test == KG_GRADIENT) return;
	if (test == KG_WAVE13PT) { t = a[0]; a[0] = a[1]; a[1] = a[2]; a[2] = t; return; }
	t = a[0]; a[0] = a[1]; a[1] = t;
}

int main(int argc, char* argv[])
{
	const int test = kgh_test_id(KG_TEST_NAME);
	const int is2d = kg_stencil_is2d(test);
	if (test < 0) { fprintf(stderr, "unknown test %s\n", KG_TEST_NAME); return 1; }
	if (argc != (is2d ? 4 : 5)) {
		if (is2d) printf("Usage: %s <nx> <ny> <nt>\n", argv[0]);
		else printf("Usage: %s <nx> <ny> <ns> <nt>\n", argv[0]);
		exit(1);
	}
	const char* no_timing = getenv("NO_TIMING");
	const char* prof_name = getenv("PROFILING_FNAME");
	const kg_dtype dt = parse_prec(getenv("B200_PREC"));
	const int variant = parse_init(getenv("B200_INIT"));
	const char* mode = getenv("B200_MODE");
	const int engine = parse_engine(getenv("B200_ENGINE"));
	const int graph = mode && !strcmp(mode, "graph");
	if (dt == KG_U8 && test != KG_GAMEOFLIFE) { fprintf(stderr, "B200_PREC=u8 is for gameoflife only\n"); exit(1); }

	const int nx = parse_arg("nx", argv[1]);
	const int ny = parse_arg("ny", argv[2]);
	const int ns = is2d ? 1 : parse_arg("ns", argv[3]);
	const int nt = parse_arg("nt", argv[is2d ? 3 : 4]);

	const int narr = kg_stencil_narrays(test);
	const size_t n = (size_t)nx * ny * ns;
	const size_t szb64 = n * sizeof(double);
	const size_t es = (dt == KG_F64 || dt == KG_F64_FMA || dt == KG_F64_FF || dt == KG_F64_MIX) ? 8 : (dt == KG_F32) ? 4 : (dt == KG_U8) ? 1 : 2;
	const size_t szb = n * es;

	double coef[6];
	double* h[6] = {0};
	for (int q = 0; q < narr; q++) {
		h[q] = (double*)memalign(MEMALIGN, szb64 ? szb64 : 8);
		if (!h[q]) { printf("Error allocating memory for arrays\n"); exit(1); }
	}
	kgh_init(test, nx, ny, ns, variant, 1u, coef, h);
	kgh_print_coefs(test, coef);
	/* wave13pt, jacobi, gaussblur, gameoflife print it unconditionally
	 * (wave13pt/wave13pt.c:756, jacobi/main.c:115, gaussblur/gaussblur.c:163,
	 * gameoflife/gameoflife.c:152). */
	const int imean_always = test == KG_WAVE13PT || test == KG_JACOBI ||
		test == KG_GAUSSBLUR || test == KG_GAMEOFLIFE;
	if (!no_timing || imean_always) printf("initial mean = %f\n", kgh_initial_mean(test, n, h));

	struct timespec t0, t1;

	/* 1) init */
	kgh_get_time(&t0);
	int count = 0;
	CU_CHECK(cudaGetDeviceCount(&count));
	KG_CHECK(kg_device_check());
	kgh_get_time(&t1);
	if (!no_timing) printf("init time = %f sec\n", kgh_time_diff(&t0, &t1));

	/* 2) alloc (plus one FP64 staging buffer when the storage type is narrower) */
	kgh_get_time(&t0);
	void* d[6] = {0};
	double* stage = NULL;
	for (int q = 0; q < narr; q++) CU_CHECK(cudaMalloc(&d[q], szb ? szb : 8));
	if (es != 8) CU_CHECK(cudaMalloc((void**)&stage, szb64 ? szb64 : 8));
	double* dsum = NULL;
	CU_CHECK(cudaMalloc((void**)&dsum, sizeof(double)));
	kgh_get_time(&t1);
	if (!no_timing) printf("device buffer alloc time = %f sec\n", kgh_time_diff(&t0, &t1));

	/* 3) load */
	kgh_get_time(&t0);
	for (int q = 0; q < narr; q++) {
		if (es == 8) {
			CU_CHECK(cudaMemcpy(d[q], h[q], szb64, cudaMemcpyHostToDevice));
		} else {
			CU_CHECK(cudaMemcpy(stage, h[q], szb64, cudaMemcpyHostToDevice));
			KG_CHECK(kg_convert(dt, d[q], KG_F64, stage, n, 0));
		}
	}
	CU_CHECK(cudaDeviceSynchronize());
	kgh_get_time(&t1);
	double load_t = kgh_time_diff(&t0, &t1);
	if (!no_timing) printf("data load time = %f sec (%f GB/sec)\n", load_t,
		narr * szb64 / (load_t * 1024 * 1024 * 1024));

	/* 4) compute */
	kg_problem p;
	memset(&p, 0, sizeof(p));
	p.stencil = test;
	p.dtype = dt;
	p.engine = engine;
	p.nx = nx;
	p.ny = is2d ? ny : ny;
	p.ns = ns;
	for (int q = 0; q < 6; q++) p.coef[q] = coef[q];
	for (int q = 0; q < narr; q++) p.arr[q] = d[q];

	if (prof_name) {
		int nregs = 0;
		KG_CHECK(kg_kernel_regcount(test, dt, &nregs));
		printf("%s regcount = %d\n", prof_name, nregs);
	}
	cudaEvent_t* ev = (cudaEvent_t*)malloc(sizeof(cudaEvent_t) * (2 * (size_t)nt + 2));
	for (int it = 0; it < 2 * nt; it++) CU_CHECK(cudaEventCreate(&ev[it]));
	kg_plan plan = NULL;
	if (graph && nt > 0) KG_CHECK(kg_plan_create(&plan, &p, nt));

	double* host_krn = (double*)calloc(nt > 0 ? (size_t)nt : 1, sizeof(double));
	if (!host_krn) { printf("Error allocating memory for timings\n"); exit(1); }
	kgh_get_time(&t0);
	if (plan) {
		CU_CHECK(cudaEventRecord(ev[0], 0));
		KG_CHECK(kg_plan_launch(plan, 0));
		CU_CHECK(cudaEventRecord(ev[1], 0));
		KG_CHECK(kg_plan_final_roles(plan, &p));
	} else {
		for (int it = 0; it < nt; it++) {
			struct timespec k0, k1;
			kgh_get_time(&k0);
			CU_CHECK(cudaEventRecord(ev[2 * it], 0));
			KG_CHECK(kg_sweep(&p, 0));
			CU_CHECK(cudaEventRecord(ev[2 * it + 1], 0));
			CU_CHECK(cudaDeviceSynchronize());
			kgh_get_time(&k1);
			host_krn[it] = kgh_time_diff(&k0, &k1);
			rotate(test, p.arr);
		}
	}
	CU_CHECK(cudaDeviceSynchronize());
	kgh_get_time(&t1);
	const double compute_t = kgh_time_diff(&t0, &t1);
	/* a TMA-engine sweep whose bounded wait gave up left its output incomplete */
	KG_CHECK(kg_engine_status(0));
	if (prof_name && !plan) {
		for (int it = 0; it < nt; it++) {
			float ms = 0;
			CU_CHECK(cudaEventElapsedTime(&ms, ev[2 * it], ev[2 * it + 1]));
			printf("%s kernel time = %f\n", prof_name, host_krn[it]);
			printf("%s device time = %f\n", prof_name, ms * 1e-3);
		}
	} else if (prof_name && nt > 0) {
		float ms = 0;
		CU_CHECK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
		printf("%s kernel time = %f\n", prof_name, compute_t / nt);
		printf("%s device time = %f\n", prof_name, ms * 1e-3 / nt);
	}
	free(host_krn);
	if (!no_timing) printf("compute time = %f sec\n", compute_t);
	for (int it = 0; it < 2 * nt; it++) cudaEventDestroy(ev[it]);
	free(ev);
	if (plan) kg_plan_destroy(plan);

	/* Final checksum on the GPU in FP64: the reference's "final mean" buffer
	 * (laplacian/laplacian.c:374-377; divergence: u; gradient: ux+uy+uz). */
	const void* fin[3];
	int nfin = 1;
	if (test == KG_GRADIENT) { fin[0] = p.arr[1]; fin[1] = p.arr[2]; fin[2] = p.arr[3]; nfin = 3; }
	else if (test == KG_DIVERGENCE) fin[0] = p.arr[0];
	else fin[0] = p.arr[1];
	KG_CHECK(kg_checksum(dt, n, nfin, fin, dsum, 0));

	/* 5) save: the result arrays back to the host */
	kgh_get_time(&t0);
	double sum = 0;
	CU_CHECK(cudaMemcpy(&sum, dsum, sizeof(double), cudaMemcpyDeviceToHost));
	for (int q = 0; q < nfin; q++) {
		if (es == 8) {
			CU_CHECK(cudaMemcpy(h[q], fin[q], szb64, cudaMemcpyDeviceToHost));
		} else {
			KG_CHECK(kg_convert(KG_F64, stage, dt, fin[q], n, 0));
			CU_CHECK(cudaMemcpy(h[q], stage, szb64, cudaMemcpyDeviceToHost));
		}
	}
	kgh_get_time(&t1);
	double save_t = kgh_time_diff(&t0, &t1);
	if (!no_timing) printf("data save time = %f sec (%f GB/sec)\n", save_t,
		nfin * szb64 / (save_t * 1024 * 1024 * 1024));

	/* 6) free */
	kgh_get_time(&t0);
	for (int q = 0; q < narr; q++) CU_CHECK(cudaFree(d[q]));
	if (stage) CU_CHECK(cudaFree(stage));
	CU_CHECK(cudaFree(dsum));
	kgh_get_time(&t1);
	if (!no_timing) printf("device buffer free time = %f sec\n", kgh_time_diff(&t0, &t1));

	printf("final mean = %f\n", n ? sum / n / nfin : 0.0);

	for (int q = 0; q < narr; q++) free(h[q]);
	fflush(stdout);
	return 0;
}
