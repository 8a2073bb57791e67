// kg_runtime.cu -- whole test programs on host arrays, and CUDA-graph plans
// of the nt-sweep time loop.
#include <chrono>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>

#include "kg_internal.h"

namespace kg {
kg_status sweep_checked(const kg_problem* p, cudaStream_t st);
kg_status validate_problem(const kg_problem* p);
const char* stencil_name(int s);

// Pointer rotation after one sweep, as the reference loops do it:
// two-buffer swap (laplacian/laplacian.c:299-300), wave13pt's three-level
// rotation (wave13pt/wave13pt.c:919), none for divergence and gradient
// (divergence/divergence.c:297-309, gradient/gradient.c:303-315).
template <class T> void rotate_roles(int stencil, T* a)
{
	if (stencil == KG_DIVERGENCE || stencil == KG_GRADIENT) return;
	if (stencil == KG_WAVE13PT) {
		T t = a[0]; a[0] = a[1]; a[1] = a[2]; a[2] = t;
		return;
	}
	T t = a[0]; a[0] = a[1]; a[1] = t;
}

static double now_s()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}


// Device memory of kg_program_run (and of kg_matmul_tc's workspace): one
// stream-ordered pool per device, owned by the library.  Allocating and freeing on the stream keeps programs that
// run concurrently on different streams from waiting on each other (cudaFree
// waits for the whole device); up to kPoolKeep bytes stay cached between
// calls (room for two concurrent tricubic programs of 512x256x256 with their
// weight planes), the rest goes back to the device when a stream synchronises.
constexpr uint64_t kPoolKeep = 48ull << 30;

cudaError_t program_pool(cudaMemPool_t* out)
{
	static std::mutex m;
	static cudaMemPool_t pools[64];
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return e;
	if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
	std::lock_guard<std::mutex> g(m);
	if (!pools[dev]) {
		cudaMemPoolProps props;
		memset(&props, 0, sizeof(props));
		props.allocType = cudaMemAllocationTypePinned;
		props.location.type = cudaMemLocationTypeDevice;
		props.location.id = dev;
		cudaMemPool_t pool;
		if ((e = cudaMemPoolCreate(&pool, &props)) != cudaSuccess) return e;
		uint64_t keep = kPoolKeep;
		if ((e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess) {
			cudaMemPoolDestroy(pool);
			return e;
		}
		pools[dev] = pool;
	}
	*out = pools[dev];
	return cudaSuccess;
}
}  // namespace kg

using namespace kg;

struct kg_plan_s {
	kg_problem p;
	int nt;
	int perm[6];   // final role q is held by original array perm[q]
	cudaGraph_t graph;
	cudaGraphExec_t exec;
	double* pw;    // tricubic: the loop-invariant weight planes (owned)
};

namespace kg {
// Whether a tricubic program takes the precomputed-weight path: the planes
// must leave at least half of the free device memory free.
static bool pw_fits(size_t bytes)
{
	if (!bytes) return false;
	size_t fr = 0, tot = 0;
	if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { cudaGetLastError(); return false; }
	return bytes <= fr / 2;
}
}  // namespace kg

extern "C" {

kg_status kg_program_run(kg_problem* p, int nt, int copy_back_mask, kg_timings* tm, kg_stream_t stream)
{
	clear_error();
	if (!p || nt < 0) return fail(KG_EINVAL, "kg_program_run: bad argument");
	const int narr = kg_stencil_narrays(p->stencil);
	if (narr < 0) return fail(KG_EINVAL, "kg_program_run: unknown stencil %d", p->stencil);
	const size_t es = dtype_size(p->dtype);
	if (es == 0) return fail(KG_EINVAL, "kg_program_run: unknown dtype %d", p->dtype);
	if (p->nx < 0 || p->ny < 0 || p->ns < 0) return fail(KG_EINVAL, "kg_program_run: negative size");
	const size_t n = (size_t)p->nx * p->ny * p->ns;
	const size_t bytes = n * es;
	for (int q = 0; q < narr; q++)
		if (!p->arr[q] && n) return fail(KG_EINVAL, "kg_program_run: host array %d is null", q);
	cudaStream_t st = (cudaStream_t)stream;
	kg_timings t;
	memset(&t, 0, sizeof(t));
	cudaMemPool_t pool;
	kg_status s = fail_cuda(program_pool(&pool), "kg_program_run: memory pool");
	if (s != KG_OK) return s;

	// Every phase is ordered on the stream and the host waits once, at the
	// end; phase times come from events between the phases.
	const int nev = 2 * nt + 6;
	cudaEvent_t* ev = new (std::nothrow) cudaEvent_t[nev];
	if (!ev) return fail(KG_ENOMEM, "kg_program_run: events");
	int made = 0;
	for (; made < nev; made++)
		if ((s = fail_cuda(cudaEventCreate(&ev[made]), "kg_program_run: events")) != KG_OK) break;
	cudaEvent_t *load0 = ev, *load1 = ev + 1, *save0 = ev + 2, *save1 = ev + 3, *free1 = ev + 4,
		*sweep = ev + 6;

	void* dev[6] = {0};
	kg_problem d = *p;
	int ran = 0;
	if (s == KG_OK) {
		const double t0 = now_s();
		for (int q = 0; q < narr && s == KG_OK; q++) {
			s = fail_cuda(cudaMallocFromPoolAsync(&dev[q], bytes ? bytes : 1, pool, st), "kg_program_run: alloc");
			d.arr[q] = dev[q];
		}
		t.alloc = now_s() - t0;
	}
	if (s == KG_OK) {
		cudaEventRecord(*load0, st);
		for (int q = 0; q < narr && s == KG_OK; q++)
			s = fail_cuda(cudaMemcpyAsync(dev[q], p->arr[q], bytes, cudaMemcpyHostToDevice, st), "kg_program_run: load");
		cudaEventRecord(*load1, st);
	}
	// tricubic: the loop-invariant weight planes once (part of the compute
	// phase), then sweeps that read them
	double* pw = nullptr;
	if (s == KG_OK && nt > 0 && (s = validate_problem(&d)) == KG_OK && pw_fits(tricubic_pw_bytes(d))) {
		if (cudaMallocFromPoolAsync((void**)&pw, tricubic_pw_bytes(d), pool, st) != cudaSuccess) {
			cudaGetLastError();
			pw = nullptr;
		}
		if (pw) s = fail_cuda(tricubic_pw_precompute(d, pw, st), "kg_program_run: tricubic weights");
	}
	for (int it = 0; it < nt && s == KG_OK; it++) {
		cudaEventRecord(sweep[2 * it], st);
		if ((s = pw ? fail_cuda(tricubic_pw_sweep(d, pw, st), "kg_program_run: tricubic")
		            : sweep_checked(&d, st)) != KG_OK) break;
		cudaEventRecord(sweep[2 * it + 1], st);
		rotate_roles(p->stencil, d.arr);
		rotate_roles(p->stencil, p->arr);
		ran++;
	}
	if (s == KG_OK) {
		cudaEventRecord(*save0, st);
		for (int q = 0; q < narr && s == KG_OK; q++) {
			if (!((copy_back_mask >> q) & 1)) continue;
			s = fail_cuda(cudaMemcpyAsync(p->arr[q], d.arr[q], bytes, cudaMemcpyDeviceToHost, st), "kg_program_run: save");
		}
		cudaEventRecord(*save1, st);
	}
	if (pw) cudaFreeAsync(pw, st);
	for (int q = 0; q < narr; q++)
		if (dev[q]) cudaFreeAsync(dev[q], st);
	if (made == nev) cudaEventRecord(*free1, st);
	const kg_status sync = fail_cuda(cudaStreamSynchronize(st), "kg_program_run");
	if (s == KG_OK) s = sync;
	// a TMA-engine sweep whose bounded wait gave up left its output incomplete
	if (s == KG_OK && ran) s = kg_engine_status(stream);
	if (s == KG_OK) {
		float ms = 0;
		cudaEventElapsedTime(&ms, *load0, *load1);
		t.load = ms * 1e-3;
		cudaEventElapsedTime(&ms, *load1, *save0);
		t.compute = ms * 1e-3;
		cudaEventElapsedTime(&ms, *save0, *save1);
		t.save = ms * 1e-3;
		cudaEventElapsedTime(&ms, *save1, *free1);
		t.free_ = ms * 1e-3;
		double sum = 0, mn = 1e30;
		for (int it = 0; it < ran; it++) {
			cudaEventElapsedTime(&ms, sweep[2 * it], sweep[2 * it + 1]);
			sum += ms * 1e-3;
			if (ms * 1e-3 < mn) mn = ms * 1e-3;
		}
		if (ran) {
			t.kernel_avg = sum / ran;
			t.kernel_min = mn;
		}
		kg_kernel_regcount(p->stencil, (kg_dtype)p->dtype, &t.nregs);
		t.weights_once = pw ? 1 : 0;
	}
	for (int i = 0; i < made; i++) cudaEventDestroy(ev[i]);
	delete[] ev;
	if (tm) *tm = t;
	return s;
}

kg_status kg_plan_create(kg_plan* plan, const kg_problem* p, int nt)
{
	clear_error();
	if (!plan || !p || nt < 1) return fail(KG_EINVAL, "kg_plan_create: bad argument");
	*plan = nullptr;
	kg_plan_s* pl = new (std::nothrow) kg_plan_s();
	if (!pl) return fail(KG_ENOMEM, "kg_plan_create");
	pl->p = *p;
	pl->nt = nt;
	for (int q = 0; q < 6; q++) pl->perm[q] = q;
	cudaStream_t cs;
	kg_status s = fail_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "kg_plan_create");
	if (s != KG_OK) { delete pl; return s; }
	kg_problem d = *p;
	// tricubic: the weight planes once, then nt sweeps that read them
	if ((s = validate_problem(p)) == KG_OK && pw_fits(tricubic_pw_bytes(*p))) {
		if (cudaMalloc((void**)&pl->pw, tricubic_pw_bytes(*p)) != cudaSuccess) {
			cudaGetLastError();
			pl->pw = nullptr;
		}
	}
	if (s == KG_OK) s = fail_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "kg_plan_create: capture");
	if (s == KG_OK) {
		if (pl->pw) s = fail_cuda(tricubic_pw_precompute(d, pl->pw, cs), "kg_plan_create: tricubic weights");
		for (int it = 0; it < nt && s == KG_OK; it++) {
			s = pl->pw ? fail_cuda(tricubic_pw_sweep(d, pl->pw, cs), "kg_plan_create: tricubic")
			           : sweep_checked(&d, cs);
			rotate_roles(p->stencil, d.arr);
			rotate_roles(p->stencil, pl->perm);
		}
		cudaGraph_t g = nullptr;
		cudaError_t e = cudaStreamEndCapture(cs, &g);
		if (s == KG_OK) s = fail_cuda(e, "kg_plan_create: end capture");
		if (s == KG_OK) {
			pl->graph = g;
			s = fail_cuda(cudaGraphInstantiate(&pl->exec, g, 0), "kg_plan_create: instantiate");
		} else if (g) {
			cudaGraphDestroy(g);
		}
	}
	cudaStreamDestroy(cs);
	if (s != KG_OK) {
		if (pl->exec) cudaGraphExecDestroy(pl->exec);
		if (pl->graph) cudaGraphDestroy(pl->graph);
		if (pl->pw) cudaFree(pl->pw);
		delete pl;
		return s;
	}
	*plan = pl;
	return KG_OK;
}

kg_status kg_plan_launch(kg_plan plan, kg_stream_t stream)
{
	clear_error();
	if (!plan) return fail(KG_EINVAL, "kg_plan_launch: null plan");
	return fail_cuda(cudaGraphLaunch(plan->exec, (cudaStream_t)stream), "kg_plan_launch");
}

kg_status kg_plan_final_roles(kg_plan plan, kg_problem* p)
{
	clear_error();
	if (!plan || !p) return fail(KG_EINVAL, "kg_plan_final_roles: bad argument");
	*p = plan->p;
	for (int q = 0; q < 6; q++) p->arr[q] = plan->p.arr[plan->perm[q]];
	return KG_OK;
}

int kg_plan_kernels(kg_plan plan)
{
	if (!plan || !plan->graph) return -1;
	size_t n = 0;
	if (cudaGraphGetNodes(plan->graph, nullptr, &n) != cudaSuccess) return -1;
	cudaGraphNode_t* nodes = new (std::nothrow) cudaGraphNode_t[n ? n : 1];
	if (!nodes) return -1;
	int k = 0;
	if (cudaGraphGetNodes(plan->graph, nodes, &n) == cudaSuccess)
		for (size_t i = 0; i < n; i++) {
			cudaGraphNodeType t;
			if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
		}
	delete[] nodes;
	return k;
}

kg_status kg_plan_destroy(kg_plan plan)
{
	clear_error();
	if (!plan) return KG_OK;
	if (plan->exec) cudaGraphExecDestroy(plan->exec);
	if (plan->graph) cudaGraphDestroy(plan->graph);
	if (plan->pw) cudaFree(plan->pw);
	delete plan;
	return KG_OK;
}

}  // extern "C"
