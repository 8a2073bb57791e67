// kg_api.cu -- the C ABI: argument checks, dispatch by storage type, errors.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <cstdint>

#include "kg_internal.h"

#ifndef KG_FF_STAGED
#define KG_FF_STAGED 0
#endif

namespace kg {

static thread_local char g_err[512];

void clear_error() { g_err[0] = 0; }

kg_status fail(kg_status s, const char* fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_err, sizeof(g_err), fmt, ap);
	va_end(ap);
	return s;
}

kg_status fail_cuda(cudaError_t e, const char* what)
{
	if (e == cudaSuccess) return KG_OK;
	if (e == cudaErrorMemoryAllocation) {
		cudaGetLastError();
		return fail(KG_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
	}
	return fail(KG_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

size_t dtype_size(int dt)
{
	switch (dt) {
	case KG_F64: case KG_F64_FMA: case KG_F64_FF: case KG_F64_MIX: return 8;
	case KG_F32: return 4;
	case KG_BF16: case KG_F16: return 2;
	case KG_U8: return 1;
	default: return 0;
	}
}

// Per stencil: arrays, coefficients, 2D, output mask (bits over arr[]).
struct Meta { int narr, ncoef, is2d, outmask; const char* name; };
static const Meta k_meta[KG_NSTENCILS] = {
	{2, 2, 0, 0x2, "laplacian"},   {4, 3, 0, 0x1, "divergence"}, {4, 3, 0, 0xE, "gradient"},
	{6, 2, 0, 0x2, "uxx1"},        {3, 3, 0, 0x4, "wave13pt"},   {5, 0, 0, 0x2, "tricubic"},
	{5, 0, 0, 0x2, "tricubic2"},   {2, 3, 1, 0x2, "jacobi"},     {2, 4, 0, 0x2, "lapgsrb"},
	{2, 6, 1, 0x2, "gaussblur"},   {2, 0, 1, 0x2, "gameoflife"},
};

// Engines built per storage type, bit e = kg_engine e (kg_dispatch.cuh).
static int engines_built(int dt)
{
	const int d = 1 << KG_ENGINE_DIRECT, st = 1 << KG_ENGINE_STAGED, t = 1 << KG_ENGINE_TMA,
		tv = 1 << KG_ENGINE_TMA_VEC;
	switch (dt) {
	case KG_F64: case KG_F64_FMA: return d | t;
	case KG_F64_FF: return st | t;
	case KG_F32: case KG_BF16: case KG_F16: return d | t | tv | (KG_FF_STAGED ? st : 0);
	case KG_U8: case KG_F64_MIX: return d;
	default: return 0;
	}
}

static bool overlaps(const void* a, const void* b, size_t bytes)
{
	const char* x = (const char*)a;
	const char* y = (const char*)b;
	return x < y + bytes && y < x + bytes;
}

static kg_status validate(const kg_problem* p)
{
	if (!p) return fail(KG_EINVAL, "null problem");
	if (p->stencil < 0 || p->stencil >= KG_NSTENCILS) return fail(KG_EINVAL, "unknown stencil %d", p->stencil);
	const Meta& m = k_meta[p->stencil];
	if (p->dtype < KG_F64 || p->dtype > KG_F64_MIX) return fail(KG_EINVAL, "%s: unknown dtype %d", m.name, p->dtype);
	if (p->dtype == KG_F64_MIX && p->stencil != KG_UXX1 && p->stencil != KG_WAVE13PT)
		return fail(KG_ENOTSUP, "%s: the FP64-state / FP32-increment form is provided for uxx1 and wave13pt", m.name);
	if (p->dtype == KG_U8 && p->stencil != KG_GAMEOFLIFE)
		return fail(KG_ENOTSUP, "%s: byte cells are provided for gameoflife only", m.name);
	if (p->nx < 0 || p->ny < 0 || p->ns < 0) return fail(KG_EINVAL, "%s: negative size", m.name);
	if (p->engine < KG_ENGINE_AUTO || p->engine > KG_ENGINE_TMA_VEC)
		return fail(KG_EINVAL, "%s: unknown engine %d", m.name, p->engine);
	if (p->engine != KG_ENGINE_AUTO && !((engines_built(p->dtype) >> p->engine) & 1))
		return fail(KG_ENOTSUP, "%s: engine %d is not built for dtype %d", m.name, p->engine, p->dtype);
	if (m.is2d && p->ns != 1) return fail(KG_EINVAL, "%s: 2D stencil needs ns == 1", m.name);
	const size_t n = (size_t)p->nx * (size_t)p->ny * (size_t)p->ns;
	if (n == 0) return KG_OK;
	if (n > ((size_t)1 << 40)) return fail(KG_EINVAL, "%s: %zu points is beyond the supported size", m.name, n);
	const size_t bytes = n * dtype_size(p->dtype);
	for (int q = 0; q < m.narr; q++)
		if (!p->arr[q]) return fail(KG_EINVAL, "%s: array %d is null", m.name, q);
	if (p->engine == KG_ENGINE_TMA || p->engine == KG_ENGINE_TMA_VEC) {
		bool aligned = ((size_t)p->nx * dtype_size(p->dtype)) % 16 == 0;
		for (int q = 0; q < m.narr; q++) aligned = aligned && (uintptr_t)p->arr[q] % 16 == 0;
		if (!aligned) return fail(KG_EINVAL, "%s: the TMA engines need 16-byte aligned arrays and rows", m.name);
	}
	// Outputs must not overlap any other array (a sweep reads its inputs while
	// writing its outputs from other threads).
	for (int q = 0; q < m.narr; q++) {
		if (!((m.outmask >> q) & 1)) continue;
		for (int r = 0; r < m.narr; r++)
			if (r != q && overlaps(p->arr[q], p->arr[r], bytes))
				return fail(KG_EINVAL, "%s: output array %d overlaps array %d", m.name, q, r);
	}
	return KG_OK;
}

static cudaError_t dispatch(const kg_problem& p, cudaStream_t st)
{
	switch (p.dtype) {
	case KG_F64: return sweep_f64(p, st);
	case KG_F64_FMA: return sweep_f64fma(p, st);
	case KG_F64_FF: return sweep_f64ff(p, st);
	case KG_F32: return sweep_f32(p, st);
	case KG_BF16: return sweep_bf16(p, st);
	case KG_F16: return sweep_f16(p, st);
	case KG_U8: return sweep_u8(p, st);
	case KG_F64_MIX: return p.stencil == KG_WAVE13PT ? sweep_wave13pt_mix(p, st) : sweep_uxx1_mix(p, st);
	default: return cudaErrorInvalidValue;
	}
}

kg_status validate_problem(const kg_problem* p) { return validate(p); }

kg_status sweep_checked(const kg_problem* p, cudaStream_t st)
{
	kg_status s = validate(p);
	if (s != KG_OK) return s;
	if ((size_t)p->nx * p->ny * p->ns == 0) return KG_OK;
	return fail_cuda(dispatch(*p, st), k_meta[p->stencil].name);
}

const char* stencil_name(int s) { return (s >= 0 && s < KG_NSTENCILS) ? k_meta[s].name : "?"; }

}  // namespace kg

using namespace kg;

extern "C" {

int kg_stencil_narrays(int s) { return (s >= 0 && s < KG_NSTENCILS) ? k_meta[s].narr : -1; }
int kg_stencil_ncoefs(int s) { return (s >= 0 && s < KG_NSTENCILS) ? k_meta[s].ncoef : -1; }
int kg_stencil_is2d(int s) { return (s >= 0 && s < KG_NSTENCILS) ? k_meta[s].is2d : -1; }
int kg_stencil_outputs(int s) { return (s >= 0 && s < KG_NSTENCILS) ? k_meta[s].outmask : 0; }

kg_status kg_sweep(const kg_problem* p, kg_stream_t stream)
{
	clear_error();
	return sweep_checked(p, (cudaStream_t)stream);
}

static kg_problem mk(int stencil, kg_dtype dt, int nx, int ny, int ns)
{
	kg_problem p;
	memset(&p, 0, sizeof(p));
	p.stencil = stencil;
	p.dtype = dt;
	p.nx = nx;
	p.ny = ny;
	p.ns = ns;
	return p;
}

kg_status kg_laplacian(kg_dtype dt, int nx, int ny, int ns, double alpha, double beta,
	const void* w0, void* w1, kg_stream_t stream)
{
	kg_problem p = mk(KG_LAPLACIAN, dt, nx, ny, ns);
	p.coef[0] = alpha; p.coef[1] = beta;
	p.arr[0] = (void*)w0; p.arr[1] = w1;
	return kg_sweep(&p, stream);
}

kg_status kg_divergence(kg_dtype dt, int nx, int ny, int ns, double alpha, double beta, double gamma,
	void* u, const void* ux, const void* uy, const void* uz, kg_stream_t stream)
{
	kg_problem p = mk(KG_DIVERGENCE, dt, nx, ny, ns);
	p.coef[0] = alpha; p.coef[1] = beta; p.coef[2] = gamma;
	p.arr[0] = u; p.arr[1] = (void*)ux; p.arr[2] = (void*)uy; p.arr[3] = (void*)uz;
	return kg_sweep(&p, stream);
}

kg_status kg_gradient(kg_dtype dt, int nx, int ny, int ns, double alpha, double beta, double gamma,
	const void* u, void* ux, void* uy, void* uz, kg_stream_t stream)
{
	kg_problem p = mk(KG_GRADIENT, dt, nx, ny, ns);
	p.coef[0] = alpha; p.coef[1] = beta; p.coef[2] = gamma;
	p.arr[0] = (void*)u; p.arr[1] = ux; p.arr[2] = uy; p.arr[3] = uz;
	return kg_sweep(&p, stream);
}

kg_status kg_uxx1(kg_dtype dt, int nx, int ny, int ns, double c1, double c2,
	const void* u0, void* u1, const void* d1, const void* xx, const void* xy, const void* xz,
	kg_stream_t stream)
{
	kg_problem p = mk(KG_UXX1, dt, nx, ny, ns);
	p.coef[0] = c1; p.coef[1] = c2;
	p.arr[0] = (void*)u0; p.arr[1] = u1; p.arr[2] = (void*)d1;
	p.arr[3] = (void*)xx; p.arr[4] = (void*)xy; p.arr[5] = (void*)xz;
	return kg_sweep(&p, stream);
}

kg_status kg_wave13pt(kg_dtype dt, int nx, int ny, int ns, double m0, double m1, double m2,
	const void* w0, const void* w1, void* w2, kg_stream_t stream)
{
	kg_problem p = mk(KG_WAVE13PT, dt, nx, ny, ns);
	p.coef[0] = m0; p.coef[1] = m1; p.coef[2] = m2;
	p.arr[0] = (void*)w0; p.arr[1] = (void*)w1; p.arr[2] = w2;
	return kg_sweep(&p, stream);
}

static kg_status tricubic_any(int stencil, kg_dtype dt, int nx, int ny, int ns,
	const void* u0, void* u1, const void* a, const void* b, const void* c, kg_stream_t stream)
{
	kg_problem p = mk(stencil, dt, nx, ny, ns);
	p.arr[0] = (void*)u0; p.arr[1] = u1; p.arr[2] = (void*)a; p.arr[3] = (void*)b; p.arr[4] = (void*)c;
	return kg_sweep(&p, stream);
}

kg_status kg_tricubic(kg_dtype dt, int nx, int ny, int ns, const void* u0, void* u1,
	const void* a, const void* b, const void* c, kg_stream_t stream)
{
	return tricubic_any(KG_TRICUBIC, dt, nx, ny, ns, u0, u1, a, b, c, stream);
}

kg_status kg_tricubic2(kg_dtype dt, int nx, int ny, int ns, const void* u0, void* u1,
	const void* a, const void* b, const void* c, kg_stream_t stream)
{
	return tricubic_any(KG_TRICUBIC2, dt, nx, ny, ns, u0, u1, a, b, c, stream);
}

kg_status kg_jacobi(kg_dtype dt, int nx, int ny, double c0, double c1, double c2,
	const void* w0, void* w1, kg_stream_t stream)
{
	kg_problem p = mk(KG_JACOBI, dt, nx, ny, 1);
	p.coef[0] = c0; p.coef[1] = c1; p.coef[2] = c2;
	p.arr[0] = (void*)w0; p.arr[1] = w1;
	return kg_sweep(&p, stream);
}

kg_status kg_lapgsrb(kg_dtype dt, int nx, int ny, int ns, double c0, double c1, double c2, double c3,
	const void* w0, void* w1, kg_stream_t stream)
{
	kg_problem p = mk(KG_LAPGSRB, dt, nx, ny, ns);
	p.coef[0] = c0; p.coef[1] = c1; p.coef[2] = c2; p.coef[3] = c3;
	p.arr[0] = (void*)w0; p.arr[1] = w1;
	return kg_sweep(&p, stream);
}

kg_status kg_gaussblur(kg_dtype dt, int nx, int ny, double s0, double s1, double s2,
	double s4, double s5, double s8, const void* w0, void* w1, kg_stream_t stream)
{
	kg_problem p = mk(KG_GAUSSBLUR, dt, nx, ny, 1);
	p.coef[0] = s0; p.coef[1] = s1; p.coef[2] = s2; p.coef[3] = s4; p.coef[4] = s5; p.coef[5] = s8;
	p.arr[0] = (void*)w0; p.arr[1] = w1;
	return kg_sweep(&p, stream);
}

kg_status kg_gameoflife(kg_dtype dt, int nx, int ny, const void* u0, void* u1, kg_stream_t stream)
{
	kg_problem p = mk(KG_GAMEOFLIFE, dt, nx, ny, 1);
	p.arr[0] = (void*)u0; p.arr[1] = u1;
	return kg_sweep(&p, stream);
}

kg_status kg_kernel_regcount(int stencil, kg_dtype dt, int* nregs)
{
	clear_error();
	if (!nregs || stencil < 0 || stencil >= KG_NSTENCILS) return fail(KG_EINVAL, "kg_kernel_regcount: bad argument");
	kg_problem p = mk(stencil, dt, 8, 8, k_meta[stencil].is2d ? 1 : 8);
	cudaError_t e;
	switch (dt) {
	case KG_F64: e = regs_f64(p, nregs); break;
	case KG_F64_FMA: e = regs_f64fma(p, nregs); break;
	case KG_F64_FF: e = regs_f64ff(p, nregs); break;
	case KG_F32: e = regs_f32(p, nregs); break;
	case KG_BF16: e = regs_bf16(p, nregs); break;
	case KG_F16: e = regs_f16(p, nregs); break;
	case KG_U8:
		if (stencil != KG_GAMEOFLIFE) return fail(KG_ENOTSUP, "byte cells: gameoflife only");
		e = regs_u8(p, nregs);
		break;
	case KG_F64_MIX:
		if (stencil != KG_UXX1 && stencil != KG_WAVE13PT)
			return fail(KG_ENOTSUP, "the FP64-state / FP32-increment form: uxx1 and wave13pt");
		e = stencil == KG_WAVE13PT ? regs_wave13pt_mix(nregs) : regs_uxx1_mix(nregs);
		break;
	default: return fail(KG_EINVAL, "kg_kernel_regcount: unknown dtype");
	}
	return fail_cuda(e, "kg_kernel_regcount");
}

int kg_sweep_launches(int stencil, kg_dtype dt)
{
	(void)dt;
	return (stencil >= 0 && stencil < KG_NSTENCILS) ? 1 : 0;
}

const char* kg_status_string(kg_status s)
{
	switch (s) {
	case KG_OK: return "KG_OK";
	case KG_EINVAL: return "KG_EINVAL";
	case KG_ECUDA: return "KG_ECUDA";
	case KG_ENOMEM: return "KG_ENOMEM";
	case KG_ETIMEOUT: return "KG_ETIMEOUT";
	case KG_ENOTSUP: return "KG_ENOTSUP";
	case KG_ENODEV: return "KG_ENODEV";
	default: return "KG_UNKNOWN";
	}
}

const char* kg_last_error(void) { return g_err; }

kg_status kg_device_check(void)
{
	clear_error();
	int n = 0;
	cudaError_t e = cudaGetDeviceCount(&n);
	if (e != cudaSuccess || n == 0) {
		cudaGetLastError();
		return fail(KG_ENODEV, "no CUDA device: %s", cudaGetErrorString(e));
	}
	cudaDeviceProp prop;
	e = cudaGetDeviceProperties(&prop, 0);
	if (e != cudaSuccess) return fail_cuda(e, "cudaGetDeviceProperties");
	if (prop.major != 10 || prop.minor != 3)
		return fail(KG_ENODEV, "device 0 is sm_%d%d, this library is built for sm_103a", prop.major, prop.minor);
	return KG_OK;
}

const char* kg_version(void) { return "kg_b200 1.0 (sm_103a)"; }

}  // extern "C"
