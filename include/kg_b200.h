/*
 * kg_b200.h -- C ABI of the GB300 (sm_103a) stencil-sweep library.
 *
 * Drop-in boundary for the kernel functions of kernelgen-perf-tests.  Each
 * kg_<test>() replaces the reference kernel of the same name: same argument
 * meaning and order, plus a storage/arithmetic type and a stream.  Pointers
 * are device pointers owned by the caller; the call borrows them, launches
 * one sweep asynchronously on `stream` and returns.  Unlike the reference
 * (CUDA_SAFE_CALL prints and exit(-1), cuda_profiling.h:11-15) nothing here
 * exits: every entry point returns a kg_status and kg_last_error() gives the
 * message.  The caller performs the ping-pong pointer swap between sweeps, as
 * the reference main() does (laplacian/laplacian.c:299-300).
 *
 * Layout: x fastest, element (i,j,k) at i + nx*j + nx*ny*k
 * (laplacian/laplacian.c:30).  2D tests take (nx, ny) with ny the full row
 * count (their makefiles pass NY*NS, gameoflife/gcc/makefile:45-46).
 *
 * Threading: calls are safe from several host threads on distinct streams;
 * a kg_plan / kg_batch object is not thread-safe.
 */
#ifndef KG_B200_H
#define KG_B200_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t; 0 is the legacy default stream. */
typedef struct CUstream_st* kg_stream_t;

typedef enum {
	KG_OK = 0,
	KG_EINVAL = 1,    /* bad argument: size, type, null or aliasing pointer */
	KG_ECUDA = 2,     /* CUDA runtime error (see kg_last_error)              */
	KG_ENOMEM = 3,    /* device or pinned-host allocation failed             */
	KG_ETIMEOUT = 4,  /* an iteration cap or a bounded device wait ran out   */
	KG_ENOTSUP = 5,   /* type not provided for this stencil                  */
	KG_ENODEV = 6     /* no sm_103 device visible                            */
} kg_status;

/* Storage type of the arrays and the arithmetic used on them. */
typedef enum {
	KG_F64 = 0,      /* FP64, reference association order, no FMA contraction:
	                    bitwise equal to an IEEE build of the reference kernel */
	KG_F64_FMA = 1,  /* FP64, products contracted into FMA where the compiler
	                    can (the suite's -ffast-math gcc build does the same)   */
	KG_F32 = 2,      /* FP32 storage and arithmetic                           */
	KG_BF16 = 3,     /* BF16 storage, FP32 arithmetic                         */
	KG_F16 = 4,      /* FP16 storage, FP32 arithmetic                         */
	KG_U8 = 5,       /* 0/1 byte cells: gameoflife only (B3/S23; other byte
	                    values give unspecified cells)                       */
	KG_F64_FF = 6,   /* FP64 storage; arithmetic on float-float pairs (hi+lo
	                    FP32 with error-free transformations) on the FP32 pipes:
	                    ~1e-14 of FP64 normwise, values within FP32's range    */
	KG_F64_MIX = 7   /* FP64 storage; the update's small part in FP32
	                    arithmetic, combined with the FP64 state in FP64 (uxx1:
	                    its increment; wave13pt: its neighbour differences from
	                    the centre): the state keeps FP64 precision, a step errs
	                    by FP32's relative error of that part.  uxx1 and
	                    wave13pt only                                          */
} kg_dtype;

/* Stencil ids (the suite's test directories). */
typedef enum {
	KG_LAPLACIAN = 0, KG_DIVERGENCE = 1, KG_GRADIENT = 2, KG_UXX1 = 3,
	KG_WAVE13PT = 4, KG_TRICUBIC = 5, KG_TRICUBIC2 = 6, KG_JACOBI = 7,
	KG_LAPGSRB = 8, KG_GAUSSBLUR = 9, KG_GAMEOFLIFE = 10, KG_NSTENCILS = 11
} kg_stencil;

/* ---- one sweep per call (device pointers, asynchronous) ---------------- */

/* laplacian/laplacian.c:44-50: w1 = alpha*w0 + beta*(6 faces), [1,n-2]^3. */
kg_status kg_laplacian(kg_dtype dt, int nx, int ny, int ns, double alpha, double beta,
	const void* w0, void* w1, kg_stream_t stream);

/* divergence/divergence.c:44-50: u is written from ux, uy, uz, [1,n-2]^3. */
kg_status kg_divergence(kg_dtype dt, int nx, int ny, int ns,
	double alpha, double beta, double gamma,
	void* u, const void* ux, const void* uy, const void* uz, kg_stream_t stream);

/* gradient/gradient.c:45-51: ux, uy, uz are written from u, [1,n-2]^3. */
kg_status kg_gradient(kg_dtype dt, int nx, int ny, int ns,
	double alpha, double beta, double gamma,
	const void* u, void* ux, void* uy, void* uz, kg_stream_t stream);

/* uxx1/uxx1.c:45-51: u1 from u0, d1, xx, xy, xz; dth = 1/nx, [2,n-2]^3. */
kg_status kg_uxx1(kg_dtype dt, int nx, int ny, int ns, double c1, double c2,
	const void* u0, void* u1, const void* d1,
	const void* xx, const void* xy, const void* xz, kg_stream_t stream);

/* wave13pt/wave13pt.c:80-86: w2 from w0, w1 (13 points), [2,n-3]^3. */
kg_status kg_wave13pt(kg_dtype dt, int nx, int ny, int ns,
	double m0, double m1, double m2,
	const void* w0, const void* w1, void* w2, kg_stream_t stream);

/* tricubic/tricubic.c:71-77: u1 from u0 and offsets a, b, c, [1,n-3]^3. */
kg_status kg_tricubic(kg_dtype dt, int nx, int ny, int ns,
	const void* u0, void* u1, const void* a, const void* b, const void* c,
	kg_stream_t stream);

/* tricubic2/tricubic2.c:38-42: same maths accumulated from 0, [2,n-3]^3. */
kg_status kg_tricubic2(kg_dtype dt, int nx, int ny, int ns,
	const void* u0, void* u1, const void* a, const void* b, const void* c,
	kg_stream_t stream);

/* jacobi/jacobi.F90:15-19 (jacobi/main.c:43-52 binds it as jacobi_):
 * 2D 9-point, 0-based interior [1,n-2]^2. */
kg_status kg_jacobi(kg_dtype dt, int nx, int ny, double c0, double c1, double c2,
	const void* w0, void* w1, kg_stream_t stream);

/* lapgsrb/lapgsrb.c:44-50: 25-point out-of-place sweep, [2,n-3]^3. */
kg_status kg_lapgsrb(kg_dtype dt, int nx, int ny, int ns,
	double c0, double c1, double c2, double c3,
	const void* w0, void* w1, kg_stream_t stream);

/* gaussblur/gaussblur.c:44-50: 2D 5x5 blur, [2,n-3]^2. */
kg_status kg_gaussblur(kg_dtype dt, int nx, int ny,
	double s0, double s1, double s2, double s4, double s5, double s8,
	const void* w0, void* w1, kg_stream_t stream);

/* gameoflife/gameoflife.c:43-48: 2D smooth Conway on real cells (KG_F64,
 * KG_F64_FMA, KG_F32) or B3/S23 on 0/1 byte cells (KG_U8), [1,n-2]^2. */
kg_status kg_gameoflife(kg_dtype dt, int nx, int ny,
	const void* u0, void* u1, kg_stream_t stream);

/* ---- the suite's other tests (not stencil sweeps) ---------------------- */
/* KG_F64 (strict IEEE, bit for bit the reference expression in its loop
 * order), KG_F64_FMA or KG_F32; device pointers; asynchronous on `stream`. */

/* vecadd/vecadd.c:38-84: w2 = w0 + w1 at every point. */
kg_status kg_vecadd(kg_dtype dt, int nx, int ny, int ns,
	const void* w0, const void* w1, void* w2, kg_stream_t stream);

/* matvec/matvec.c:37-71: y[j] = sum over i of A[i + nx*j] * x[i], summed
 * in order i = 0, 1, ... from y[j] = 0. */
kg_status kg_matvec(kg_dtype dt, int nx, int ny,
	const void* A, const void* x, void* y, kg_stream_t stream);

/* matmul/matmul.F90:14-68 (column-major, as the Fortran kernel): C(i,j) =
 * C(i,j) + A(i,k) * B(k,j) in order k = 1..ny, with A(i,k) at A[i + nx*k],
 * B(k,j) at B[k + ny*j], C(i,j) at C[i + nx*j]; C accumulates (the caller
 * sets its initial value). */
kg_status kg_matmul(kg_dtype dt, int nx, int ny, int ns,
	const void* A, const void* B, void* C, kg_stream_t stream);

/* The same C(i,j) += sum over k of A(i,k) B(k,j) on FP32 arrays (same
 * layout) on the tensor cores: each operand split into a TF32 part and an
 * exact FP32 remainder, three TF32 products per product (tcgen05 kind::tf32,
 * FP32 accumulation), then added to C.  FP32-accurate (about 1e-7 of the sum
 * of |A(i,k) B(k,j)|), not the k-ordered sum: not bit for bit with
 * kg_matmul.  Takes a workspace of 8 (nx + ns) kp bytes (kp: ny rounded up
 * to a multiple of 32) from the library's stream-ordered pool (the one
 * kg_program_run uses; its memory stays cached between calls).  KG_ENOTSUP off Blackwell; a wait that gives up is
 * reported by kg_engine_status. */
kg_status kg_matmul_tc(int nx, int ny, int ns, const float* A, const float* B, float* C, kg_stream_t stream);

/* sincos/sincos.F90:60-72: xy = sin(x) + cos(y) at every point (CUDA's
 * sin/cos: within 2 ulp of the correctly rounded values, not bitwise). */
kg_status kg_sincos(kg_dtype dt, int nx, int ny, int ns,
	const void* x, const void* y, void* xy, kg_stream_t stream);

/* whispering/whispering.c:44-108: one step on [1,nx-2] x [1,ny-2]; e holds
 * two planes (component c of (i,j) at e[i + nx*j + nx*ny*c]) and is updated
 * in place with the result of the reference's serial loop order (its ey and
 * ex terms read e already updated at (i,j-1) and (i-1,j)). */
kg_status kg_whispering(kg_dtype dt, int nx, int ny, double mu, double epsilon,
	void* e, const void* h0, void* h1, const void* u_em0, void* u_em1,
	const void* ca, const void* cb, const void* da, const void* db, kg_stream_t stream);

/* Registers per thread of the main kernel of the named test above (the one that
 * runs on 16-byte aligned arrays). */
kg_status kg_extra_regcount(const char* name, kg_dtype dt, int* nregs);

/* ---- table-driven form of the same entry points ------------------------ */

/* Which kernel design runs a sweep (kg_problem.engine).  AUTO: TMA_VEC for
 * KG_F32/KG_BF16/KG_F16 stencils (all eleven) where every array and row
 * starts on a 16-byte boundary (TMA or DIRECT otherwise); DIRECT for
 * KG_F64/KG_F64_FMA; STAGED for KG_F64_FF (TMA for its divergence and uxx1
 * where aligned).  Built: DIRECT and TMA for every floating type but
 * KG_F64_FF and KG_F64_MIX; TMA_VEC for KG_F32/KG_BF16/KG_F16; STAGED and TMA
 * for KG_F64_FF; DIRECT for KG_F64_MIX and KG_U8.  Grids of tiles beyond the
 * launch limits are taken in turn.  The engines evaluate the same
 * expressions in the same order (the tests check their outputs equal bit for
 * bit).  TMA and TMA_VEC need 16-byte aligned arrays and rows; TMA_VEC
 * sweeps are launched as programmatic dependents of the kernel before them
 * on the stream (their launch overlaps its tail; they read and write nothing
 * before it has completed). */
typedef enum {
	KG_ENGINE_AUTO = 0,
	KG_ENGINE_DIRECT = 1,   /* one thread per column, neighbours through L1     */
	KG_ENGINE_STAGED = 2,   /* halo planes in shared memory, loaded by threads  */
	KG_ENGINE_TMA = 3,      /* halo planes in shared memory by tiled bulk copy  */
	KG_ENGINE_TMA_VEC = 4   /* the same copies; each thread evaluates 4 (8)
	                           consecutive points from vector reads (3D ops
	                           along z, 2D ops down bands of rows; FP32
	                           arithmetic: KG_F32, KG_BF16, KG_F16)          */
} kg_engine;

typedef struct {
	int32_t stencil;     /* kg_stencil */
	int32_t dtype;       /* kg_dtype   */
	int32_t nx, ny, ns;  /* 2D stencils: ns = 1 */
	int32_t engine;      /* kg_engine (0 = AUTO) */
	double coef[6];      /* coefficients in the reference's argument order */
	void* arr[6];        /* arrays in the reference's argument order       */
} kg_problem;

int kg_stencil_narrays(int stencil);    /* -1 for an unknown id */
int kg_stencil_ncoefs(int stencil);
int kg_stencil_is2d(int stencil);
/* Arrays a sweep writes, as a bit mask over kg_problem.arr. */
int kg_stencil_outputs(int stencil);

/* One sweep of p (device pointers). */
kg_status kg_sweep(const kg_problem* p, kg_stream_t stream);

/* Waits for `stream`, then reports whether a TMA-engine sweep since the last
 * call gave up waiting for its tile copies (KG_ETIMEOUT: that sweep's output
 * is incomplete) and clears the record.  The record is one flag per device,
 * shared by every stream; its device address is looked up once per device
 * (do not use the library across cudaDeviceReset).  No counterpart in the
 * reference. */
kg_status kg_engine_status(kg_stream_t stream);

/* How long (GPU clock cycles) a TMA-engine compute warp waits for a step's
 * tile copies before it gives up, for kernels launched after the call
 * (plans and batches keep the limit they were recorded with).  Negative:
 * the default, 2^31 cycles (about 1 s).  0: give up unless the copies have
 * already landed when the warp first looks -- a way to make the failure
 * path run without a fault, for tests.  Whatever the limit, a CTA that
 * gives up waits for every copy it issued before it exits.  Process-wide.
 * No counterpart in the reference. */
kg_status kg_set_tma_wait_limit(long long cycles);

/* ---- checksums (the reference's "initial mean" / "final mean") ---------- */

/* out_dev[0] = sum over i of (a_0[i] + a_1[i] + ... + a_{narr-1}[i]) in FP64,
 * narr <= 6, arrays of type dt with n elements each.  Deterministic: a fixed
 * two-level tree, the same bits on every run.  Scratch (one double per block
 * of the first level) comes from the stream-ordered pool. */
kg_status kg_checksum(kg_dtype dt, size_t n, int narr, const void* const* arrays,
	double* out_dev, kg_stream_t stream);

/* kg_checksum for callers that cannot allocate device memory while they run:
 * a host framework that owns all device memory through its own arena, or a
 * latency-critical loop that cannot accept the synchronisation cudaMalloc /
 * cudaFree may cause.  Same arguments, same first/second-level tree and so
 * the same result bits as kg_checksum; no cudaMalloc, cudaFree or other
 * allocating call.  The partial sums live in a fixed device array of
 * KG_CHECKSUM_NOALLOC_PARTIALS doubles (16 KiB) that every GPU loading the
 * library keeps until the process exits; n above KG_CHECKSUM_NOALLOC_MAX_N
 * is rejected with KG_EINVAL.  The first call on each device looks up the
 * array's device address (make it before any stream capture), and with
 * CUDA's lazy module loading the first launch of each storage type's two
 * kernels loads them, which may itself take device memory and synchronise:
 * make one call per device and storage type at start-up, before the phase
 * that must not allocate.  The cached address does not survive
 * cudaDeviceReset: do not use the library across a device reset.  All calls
 * share the array: calls whose kernels may overlap on the GPU (different
 * streams without ordering) race and must be serialised by the caller.
 * No counterpart in the reference. */
#define KG_CHECKSUM_NOALLOC_PARTIALS 2048
#define KG_CHECKSUM_NOALLOC_MAX_N ((size_t)1 << 33)
kg_status kg_checksum_noalloc(kg_dtype dt, size_t n, int narr, const void* const* arrays,
	double* out_dev, kg_stream_t stream);

/* Error of a low-precision result x (type dt) against an FP64 reference:
 * out_dev[0] = max |x-ref|, [1] = sum (x-ref)^2, [2] = max |ref|,
 * [3] = sum ref^2, all in FP64. */
kg_status kg_error_stats(kg_dtype dt, size_t n, const void* x, const double* ref,
	double* out_dev, kg_stream_t stream);

/* Convert between storage types (FP64 <-> FP32/BF16/FP16, FP64 <-> U8 by
 * threshold 0.5), elementwise. */
kg_status kg_convert(kg_dtype dst_t, void* dst, kg_dtype src_t, const void* src,
	size_t n, kg_stream_t stream);

/* ---- whole test program on host arrays ---------------------------------- */

typedef struct {
	double alloc;           /* seconds on the host clock to enqueue allocs  */
	double load, compute, save, free_;  /* seconds, CUDA events on stream  */
	double kernel_avg;      /* mean device time of one sweep (CUDA events)  */
	double kernel_min;
	int nregs;              /* registers per thread of the sweep kernel     */
	int weights_once;       /* 1: tricubic's loop-invariant weight products
	                           were evaluated once for the nt sweeps        */
} kg_timings;

/* Phases 2-6 of the reference main() (laplacian/laplacian.c:222-370) for one
 * test program: allocate device arrays, copy p->arr (HOST pointers) in, run
 * nt sweeps with the reference's pointer rotation (two-buffer swap; wave13pt
 * three-level rotation; divergence and gradient no swap), copy back the
 * arrays selected by copy_back_mask (bit q = p->arr[q] in its final role),
 * free.  On return p->arr holds the host arrays in their final roles, as the
 * reference's idxs[] leaves them.  timings may be NULL.
 * Every phase is ordered on `stream` (device memory from a library-owned
 * stream-ordered pool that keeps up to 48 GiB cached between calls) and the
 * call waits for the stream once, at the end; so calls from different host
 * threads on different streams overlap one program's copies with another's
 * sweeps.  The host arrays should be pinned for the copies to overlap. */
kg_status kg_program_run(kg_problem* p, int nt, int copy_back_mask, kg_timings* timings,
	kg_stream_t stream);

/* ---- launch plans: the nt-sweep loop captured as one CUDA graph ---------- */

typedef struct kg_plan_s* kg_plan;
/* Records nt sweeps of p (device pointers) with the reference's rotation.
 * tricubic and tricubic2 in KG_F64 / KG_F64_FMA: the plan also owns 64
 * weight planes (512 bytes per point, taken when they leave half of the free
 * device memory free): each replay first evaluates the loop-invariant weight
 * products of every point once (a, b, c do not change during the loop) and
 * the nt sweeps read them; results are bit for bit those of nt kg_sweep
 * calls.  kg_program_run does the same with the planes from its pool. */
kg_status kg_plan_create(kg_plan* plan, const kg_problem* p, int nt);
kg_status kg_plan_launch(kg_plan plan, kg_stream_t stream);
/* After a launch: p->arr in their final roles. */
kg_status kg_plan_final_roles(kg_plan plan, kg_problem* p);
/* Kernel launches in one replay of the plan (-1 on a bad plan). */
int kg_plan_kernels(kg_plan plan);
kg_status kg_plan_destroy(kg_plan plan);

/* ---- batches: many uneven problems, one persistent launch per step ------ */

/* Up to 4096 independent problems of laplacian, divergence, wave13pt and
 * gaussblur (2D, ns = 1), all KG_F32 or all KG_F64, advanced together.  Each
 * launch is one persistent kernel over the tiles of every problem and
 * advances every problem 1 step, or T steps with temporal blocking (blocks
 * evaluated T steps deep in shared memory; the library then keeps a second
 * set of the rotating arrays, allocated when such a configuration is first
 * set, and every kg_batch_step / graph replay ends with all arrays in the
 * problems' own buffers).  Each problem's arrays rotate their roles per step
 * as the reference loops do.  Results equal nsteps kg_sweep calls per
 * problem, bit for bit, every array.
 * No counterpart in the reference (each suite program runs one problem). */
typedef struct kg_batch_s* kg_batch;
typedef struct {
	int shape, bx, by, kc;   /* temporal == 1: tile of BX*BY threads on as many
	                            consecutive (i,j) columns, KC planes each (2D:
	                            KC runs of points); temporal > 1: output block
	                            of BX x BY x KC points (2D: BX x BY*KC)     */
	int ctas_per_sm;
	int tiles;               /* tiles (blocks) of all problems per launch */
	int nshapes;             /* configurations the tuner tries */
	int temporal;            /* steps per launch (temporal-blocking factor) */
	int staged;              /* 1: a tile of BX consecutive columns and KC
	                            planes whose inputs are staged in shared
	                            memory by bulk copies, one step per launch */
	int reserved;
	long long steps_done;
} kg_batch_config;
kg_status kg_batch_create(kg_batch* b, const kg_problem* probs, int nprob);
/* Launches nsteps steps on the stream. */
kg_status kg_batch_step(kg_batch b, int nsteps, kg_stream_t stream);
/* Captures nsteps steps (plus the step-counter advance) as a CUDA graph;
 * kg_batch_launch replays it and continues from the current step. */
kg_status kg_batch_capture(kg_batch b, int nsteps);
kg_status kg_batch_launch(kg_batch b, kg_stream_t stream);
/* Times every configuration -- the one-step tile shapes, the temporal
 * blocks with their factors T = 2, 3, 4 and the bulk-staged tiles -- with as
 * many CTAs per SM as stay resident, one fewer, half as many, twice and four
 * times as many (up to 32), on this batch (advancing it), and keeps the
 * fastest; cache_path (may be NULL) stores and reuses the choice per device,
 * problem list and configuration table. */
kg_status kg_batch_tune(kg_batch b, const char* cache_path, kg_stream_t stream);
kg_status kg_batch_set_config(kg_batch b, int shape, int ctas_per_sm);
kg_status kg_batch_get_config(kg_batch b, kg_batch_config* cfg);
/* Sets the step count (roles restart from step 0 with 0). */
kg_status kg_batch_set_step(kg_batch b, long long step);
/* Problem q with its arrays in the reference's roles after the steps done. */
kg_status kg_batch_final_roles(kg_batch b, int q, kg_problem* out);
kg_status kg_batch_destroy(kg_batch b);

/* ---- Poisson solves: red-black SOR, mixed-precision iterative refinement -- */

/* A u = f with the 7-point Laplacian (A u = 6 u - sum of the 6 face
 * neighbours), u = 0 on the outer planes, f and u FP64 on the device (u holds
 * the initial guess and receives the solution).  KG_SOLVE_SOR_F64: red-black
 * SOR in FP64.  KG_SOLVE_IR_*_F32: FP64 residual and correction around FP32
 * red-black SOR or Jacobi sweeps.  Stops when ||f - A u||_2 <= rtol ||f||_2
 * (checked every sweeps_per_check sweeps) or returns KG_ETIMEOUT after
 * max_sweeps.  No counterpart in the reference (its lapgsrb is an out-of-
 * place 25-point sweep, lapgsrb/lapgsrb.c:81-117, not red-black SOR). */
enum { KG_SOLVE_SOR_F64 = 0, KG_SOLVE_IR_SOR_F32 = 1, KG_SOLVE_IR_JACOBI_F32 = 2 };
#define KG_SOLVE_HISTORY 256
typedef struct {
	int kind;
	int sweeps_per_check;
	double omega;          /* SOR relaxation factor, 0 < omega < 2 */
	double rtol;           /* relative residual target */
	long long max_sweeps;
} kg_solve_opts;
typedef struct {
	long long sweeps;      /* relaxation sweeps done (one red + one black half each) */
	int outer;             /* refinement steps (FP64 corrections) */
	int nhistory;
	double rel_residual;   /* final ||f - A u|| / ||f|| */
	double fnorm;
	double seconds;        /* host wall clock of the solve */
	long long history_sweeps[KG_SOLVE_HISTORY];
	double history_rel[KG_SOLVE_HISTORY];
} kg_solve_report;
kg_status kg_poisson_solve(int nx, int ny, int ns, const double* f, double* u,
	const kg_solve_opts* opts, kg_solve_report* report, kg_stream_t stream);

/* ---- introspection and errors ------------------------------------------ */

/* Arithmetic issue rates of the current device, measured with throughput
 * kernels (operations per second; an FMA counts as one operation).  The FP64
 * sweeps are bound by fp64_ops, the roofline denominator they report.
 * No counterpart in the reference (its roofline rule uses nvprof metrics,
 * wave13pt/cuda/makefile:57-66). */
typedef struct {
	double fp64_ops;    /* DFMA per second  */
	double fp32_ops;    /* FFMA per second  */
	double int32_ops;   /* IMAD per second  */
	int sms;
	int reserved;
} kg_peaks;
kg_status kg_measure_peaks(kg_peaks* out, kg_stream_t stream);

/* Element-wise out[i] = a[i] (op) b[i] on device arrays of n doubles, through
 * the FP64 arithmetic the KG_F64 sweeps run on the integer pipes (exact IEEE
 * round-to-nearest-even addition, multiplication and division built from
 * integer and FP32 operations: KG_ARITH_ADD/MUL/DIV) or through the FP64
 * unit (KG_ARITH_NATIVE_*), so that the former can be checked bit for bit
 * against IEEE arithmetic on any operands.  A verification entry point; no
 * counterpart in the reference. */
typedef enum {
	KG_ARITH_ADD = 0,
	KG_ARITH_MUL = 1,
	KG_ARITH_DIV = 2,
	KG_ARITH_NATIVE_ADD = 3,
	KG_ARITH_NATIVE_MUL = 4,
	KG_ARITH_NATIVE_DIV = 5
} kg_arith_op;
kg_status kg_exact_arith(int op, size_t n, const double* a, const double* b, double* out, kg_stream_t stream);

/* Registers per thread of the kernel one sweep of (stencil, dt) launches. */
kg_status kg_kernel_regcount(int stencil, kg_dtype dt, int* nregs);
/* Kernel launches one sweep of (stencil, dt) makes (for launch counting). */
int kg_sweep_launches(int stencil, kg_dtype dt);
const char* kg_status_string(kg_status s);
/* Message of the last failing call on this host thread ("" if none). */
const char* kg_last_error(void);
/* KG_OK if device 0 is an sm_103 GPU. */
kg_status kg_device_check(void);
/* Library version string. */
const char* kg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* KG_B200_H */
