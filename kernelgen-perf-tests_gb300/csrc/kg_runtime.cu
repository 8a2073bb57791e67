// kg_runtime.cu -- whole test programs on host arrays, and CUDA-graph plans
// of the nt-sweep time loop.
#include <chrono>
#include <cstring>
#include <new>

#include "kg_internal.h"

namespace kg {
kg_status sweep_checked(const kg_problem* p, cudaStream_t st);
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

}  // namespace kg

using namespace kg;

struct kg_plan_s {
	kg_problem p;
	int nt;
	int perm[6];   // final role q is held by original array perm[q]
	cudaGraph_t graph;
	cudaGraphExec_t exec;
};

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

	void* dev[6] = {0};
	kg_problem d = *p;
	kg_status s = KG_OK;
	cudaEvent_t* ev = nullptr;

	double t0 = now_s();
	for (int q = 0; q < narr; q++) {
		cudaError_t e = cudaMalloc(&dev[q], bytes ? bytes : 1);
		if (e != cudaSuccess) { s = fail_cuda(e, "kg_program_run: cudaMalloc"); goto out; }
		d.arr[q] = dev[q];
	}
	t.alloc = now_s() - t0;

	t0 = now_s();
	for (int q = 0; q < narr; q++) {
		cudaError_t e = cudaMemcpyAsync(dev[q], p->arr[q], bytes, cudaMemcpyHostToDevice, st);
		if (e != cudaSuccess) { s = fail_cuda(e, "kg_program_run: load"); goto out; }
	}
	if ((s = fail_cuda(cudaStreamSynchronize(st), "kg_program_run: load")) != KG_OK) goto out;
	t.load = now_s() - t0;

	ev = new (std::nothrow) cudaEvent_t[2 * (size_t)nt + 2];
	if (!ev) { s = fail(KG_ENOMEM, "kg_program_run: events"); goto out; }
	for (int i = 0; i < 2 * nt; i++) cudaEventCreate(&ev[i]);
	t0 = now_s();
	for (int it = 0; it < nt; it++) {
		cudaEventRecord(ev[2 * it], st);
		if ((s = sweep_checked(&d, st)) != KG_OK) break;
		cudaEventRecord(ev[2 * it + 1], st);
		rotate_roles(p->stencil, d.arr);
		rotate_roles(p->stencil, p->arr);
	}
	if (s == KG_OK) s = fail_cuda(cudaStreamSynchronize(st), "kg_program_run: compute");
	t.compute = now_s() - t0;
	if (s == KG_OK && nt > 0) {
		double sum = 0, mn = 1e30;
		for (int it = 0; it < nt; it++) {
			float ms = 0;
			cudaEventElapsedTime(&ms, ev[2 * it], ev[2 * it + 1]);
			sum += ms * 1e-3;
			if (ms * 1e-3 < mn) mn = ms * 1e-3;
		}
		t.kernel_avg = sum / nt;
		t.kernel_min = mn;
	}
	for (int i = 0; i < 2 * nt; i++) cudaEventDestroy(ev[i]);
	delete[] ev;
	if (s != KG_OK) goto out;
	kg_kernel_regcount(p->stencil, (kg_dtype)p->dtype, &t.nregs);

	t0 = now_s();
	for (int q = 0; q < narr; q++) {
		if (!((copy_back_mask >> q) & 1)) continue;
		cudaError_t e = cudaMemcpyAsync(p->arr[q], d.arr[q], bytes, cudaMemcpyDeviceToHost, st);
		if (e != cudaSuccess) { s = fail_cuda(e, "kg_program_run: save"); goto out; }
	}
	if ((s = fail_cuda(cudaStreamSynchronize(st), "kg_program_run: save")) != KG_OK) goto out;
	t.save = now_s() - t0;

out:
	t0 = now_s();
	for (int q = 0; q < narr; q++)
		if (dev[q]) cudaFree(dev[q]);
	t.free_ = now_s() - t0;
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
	s = fail_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "kg_plan_create: capture");
	if (s == KG_OK) {
		for (int it = 0; it < nt && s == KG_OK; it++) {
			s = sweep_checked(&d, cs);
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

kg_status kg_plan_destroy(kg_plan plan)
{
	clear_error();
	if (!plan) return KG_OK;
	if (plan->exec) cudaGraphExecDestroy(plan->exec);
	if (plan->graph) cudaGraphDestroy(plan->graph);
	delete plan;
	return KG_OK;
}

}  // extern "C"
