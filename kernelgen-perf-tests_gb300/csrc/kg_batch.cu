// kg_batch.cu -- many independent problems of uneven sizes and mixed stencils
// advanced together: one persistent launch per time step.
//
// Layout.  A device table holds one descriptor per problem (stencil, sizes,
// coefficients, its arrays in their original roles, its tile counts and the
// index of its first tile in the global tile list).  The launch has
// ctas_per_sm x #SMs CTAs; CTA b takes tiles b, b + gridDim.x, ... of the
// global list, finds the owning problem by binary search over the prefix
// offsets (kept in shared memory) and runs that stencil's tile body -- the
// same body the single-problem sweeps use, so every problem's result equals
// its own kg_sweep bit for bit.
//
// Roles.  Array roles rotate with the step number as the reference loops
// rotate their pointers (two-buffer swap; wave13pt's three levels; none for
// divergence).  The step number lives on the device: each launch reads the
// base and adds its position in the sequence, and a one-thread kernel after
// the sequence advances the base, so a captured N-step graph can be replayed
// and continue where it stopped.
//
// Tuning.  The tile shape (BX x BY x KC) and the CTAs per SM are chosen by
// timing every candidate on the batch itself (kg_batch_tune); the choice is
// cached in a text file keyed by the device and a hash of the problem list.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <algorithm>

// the batch's small tiles are latency-bound: every sum on the FP64 unit
#define KG_SUMS_ON_FP64_UNIT 1
#include "kg_engine.cuh"
#include "kg_internal.h"

namespace kg {

constexpr int kBatchMax = 4096;

struct BatchDesc {
	int stencil, nx, ny, ns;
	int tiles_x, tiles_y, tiles_z, first;
	double c[8];          // coefficients in the compute type's precision (as double)
	void* a[4];           // arrays in their original roles
};

// Roles of the arrays of problem d at time step `step`.
template <class S>
__device__ __forceinline__ void batch_roles(const BatchDesc& d, long long step, Ptrs<S>& p)
{
	switch (d.stencil) {
	case KG_LAPLACIAN: case KG_GAUSSBLUR: {
		const int r = (int)(step & 1);
		p.in[0] = (const S*)d.a[r];
		p.out[0] = (S*)d.a[r ^ 1];
		break;
	}
	case KG_WAVE13PT: {
		const int r = (int)(step % 3);
		p.in[0] = (const S*)d.a[r];
		p.in[1] = (const S*)d.a[(r + 1) % 3];
		p.out[0] = (S*)d.a[(r + 2) % 3];
		break;
	}
	case KG_DIVERGENCE:
	default:
		p.out[0] = (S*)d.a[0];
		p.in[0] = (const S*)d.a[1];
		p.in[1] = (const S*)d.a[2];
		p.in[2] = (const S*)d.a[3];
		break;
	}
}

// One tile of a batch problem.  The (i, j) columns of the update domain are
// numbered row by row and a tile takes NT consecutive ones (3D: each thread
// then walks KC planes of its column; 2D: KC points NT apart), so tiles of
// narrow problems are not cut at every row end: only the last tile of a
// plane runs partly idle.
template <class Op, class N, class S, int NT, int KC, int UK>
__device__ __forceinline__ void sweep_lin(const Op& op, const Ptrs<S>& p, int nx, int ny, int ns, int tcol, int tz)
{
	constexpr Slots sl = Op::slots();
	constexpr bool k2d = (Op::LZ == 0 && Op::HZ == 0);
	const int tid = threadIdx.x + threadIdx.y * blockDim.x;
	const int dxn = nx - Op::LX - Op::HX, dyn = ny - Op::LY - Op::HY;
	const long long ncol = (long long)dxn * dyn;
	const long long sy = nx, sz = (long long)nx * ny;
	if (k2d) {
#pragma unroll 1
		for (int r = 0; r < KC; r++) {
			const long long col = ((long long)tcol * KC + r) * NT + tid;
			if (col >= ncol) break;
			const int j = Op::LY + (int)(col / dxn), i = Op::LX + (int)(col - (col / dxn) * dxn);
			const long long c = i + sy * j;
			GAcc<N, S> at{p.in, c, sy, sz};
			N o[3];
			op.point(at, o);
#pragma unroll
			for (int q = 0; q < sl.nout; q++) p.out[q][c] = Conv<N, S>::to(o[q]);
		}
	} else {
		const long long col = (long long)tcol * NT + tid;
		if (col >= ncol) return;
		const int j = Op::LY + (int)(col / dxn), i = Op::LX + (int)(col - (col / dxn) * dxn);
		const int k0 = Op::LZ + tz * KC, k1 = min(k0 + KC, ns - Op::HZ);
#pragma unroll UK
		for (int k = k0; k < k1; k++) {
			const long long c = i + sy * j + sz * k;
			GAcc<N, S> at{p.in, c, sy, sz};
			N o[3];
			op.point(at, o);
#pragma unroll
			for (int q = 0; q < sl.nout; q++) p.out[q][c] = Conv<N, S>::to(o[q]);
		}
	}
}

// Registers capped for 2048 resident threads per SM (32 per thread; a few
// spill): the batch's small tiles are bound by load latency, and the extra
// warps hide it.  Measured on 256 FP32 problems (Gpts/s, best tile shape and
// CTAs per SM): 188 uncapped (40 registers, 6 CTAs of 256 threads), 282
// capped.
template <class N, class S, int BX, int BY, int KC>
__global__ void __launch_bounds__(BX * BY, 2048 / (BX * BY)) batch_kernel(const BatchDesc* __restrict__ desc, int nprob,
	int total, const long long* __restrict__ step_base, int local)
{
	constexpr int NT = BX * BY;
	__shared__ int first[kBatchMax + 1];
	for (int q = threadIdx.x + threadIdx.y * BX; q < nprob; q += BX * BY) first[q] = desc[q].first;
	__syncthreads();
	const long long step = *step_base + local;
	for (int item = blockIdx.x; item < total; item += gridDim.x) {
		int lo = 0, hi = nprob - 1;
		while (lo < hi) {
			const int mid = (lo + hi + 1) >> 1;
			if (first[mid] <= item) lo = mid;
			else hi = mid - 1;
		}
		const BatchDesc& d = desc[lo];
		const int t = item - d.first;
		const int tcol = t % d.tiles_x, tz = t / d.tiles_x;
		Ptrs<S> p{};
		batch_roles<S>(d, step, p);
		switch (d.stencil) {
		case KG_LAPLACIAN:
			sweep_lin<OpLaplacian<N>, N, S, NT, KC, 4>(OpLaplacian<N>{N(d.c[0]), N(d.c[1])}, p, d.nx, d.ny, d.ns, tcol, tz);
			break;
		case KG_DIVERGENCE:
			sweep_lin<OpDivergence<N>, N, S, NT, KC, 4>(OpDivergence<N>{N(d.c[0]), N(d.c[1]), N(d.c[2])},
				p, d.nx, d.ny, d.ns, tcol, tz);
			break;
		case KG_WAVE13PT:
			sweep_lin<OpWave13pt<N>, N, S, NT, KC, 4>(OpWave13pt<N>{N(d.c[0]), N(d.c[1]), N(d.c[2])},
				p, d.nx, d.ny, d.ns, tcol, tz);
			break;
		case KG_GAUSSBLUR:
			sweep_lin<OpGaussblur<N>, N, S, NT, KC, 4>(OpGaussblur<N>{N(d.c[0]), N(d.c[1]), N(d.c[2]),
				N(d.c[3]), N(d.c[4]), N(d.c[5]), N(d.c[6])}, p, d.nx, d.ny, d.ns, tcol, tz);
			break;
		default: break;
		}
	}
}

__global__ void batch_advance(long long* step_base, int n)
{
	if (threadIdx.x == 0 && blockIdx.x == 0) *step_base += n;
}

// Tile shapes the tuner tries (BX, BY, KC).
struct Shape { int bx, by, kc; };
static const Shape k_shapes[] = {{32, 8, 8}, {32, 4, 8}, {64, 4, 8}, {32, 8, 4}, {32, 8, 16}, {128, 2, 8},
	{32, 8, 32}, {32, 16, 16}, {32, 4, 32}, {32, 8, 64}};
static const int k_nshapes = sizeof(k_shapes) / sizeof(k_shapes[0]);

template <class N, class S>
static cudaError_t launch_shape(int shape, dim3 grid, const BatchDesc* desc, int nprob, int total,
	const long long* base, int local, cudaStream_t st)
{
	switch (shape) {
#define KG_SHAPE_CASE(I, BX, BY, KC) \
	case I: batch_kernel<N, S, BX, BY, KC><<<grid, dim3(BX, BY), 0, st>>>(desc, nprob, total, base, local); break;
	KG_SHAPE_CASE(0, 32, 8, 8)
	KG_SHAPE_CASE(1, 32, 4, 8)
	KG_SHAPE_CASE(2, 64, 4, 8)
	KG_SHAPE_CASE(3, 32, 8, 4)
	KG_SHAPE_CASE(4, 32, 8, 16)
	KG_SHAPE_CASE(5, 128, 2, 8)
	KG_SHAPE_CASE(6, 32, 8, 32)
	KG_SHAPE_CASE(7, 32, 16, 16)
	KG_SHAPE_CASE(8, 32, 4, 32)
	KG_SHAPE_CASE(9, 32, 8, 64)
#undef KG_SHAPE_CASE
	default: return cudaErrorInvalidValue;
	}
	return cudaGetLastError();
}

// Tiles of one problem for a shape: runs of bx*by columns (3D: times runs
// of kc planes; 2D: kc runs per tile).
// Resident CTAs per SM of the kernel of a shape (the persistent grid should
// not exceed one wave: a CTA that starts late runs its share of the items
// after the others have finished).
template <class N, class S>
static int shape_occupancy(int shape)
{
	int n = 0;
	switch (shape) {
#define KG_OCC_CASE(I, BX, BY, KC) \
	case I: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<N, S, BX, BY, KC>, BX * BY, 0); break;
	KG_OCC_CASE(0, 32, 8, 8)
	KG_OCC_CASE(1, 32, 4, 8)
	KG_OCC_CASE(2, 64, 4, 8)
	KG_OCC_CASE(3, 32, 8, 4)
	KG_OCC_CASE(4, 32, 8, 16)
	KG_OCC_CASE(5, 128, 2, 8)
	KG_OCC_CASE(6, 32, 8, 32)
	KG_OCC_CASE(7, 32, 16, 16)
	KG_OCC_CASE(8, 32, 4, 32)
	KG_OCC_CASE(9, 32, 8, 64)
#undef KG_OCC_CASE
	default: break;
	}
	return n > 0 ? n : 1;
}

static int tiles_of(int stencil, int nx, int ny, int ns, const Shape& s, int* tx, int* ty, int* tz)
{
	int lx, hx, ly, hy, lz, hz;
	switch (stencil) {
	case KG_LAPLACIAN: case KG_DIVERGENCE: lx = hx = ly = hy = lz = hz = 1; break;
	case KG_WAVE13PT: lx = hx = ly = hy = lz = hz = 2; break;
	case KG_GAUSSBLUR: lx = hx = ly = hy = 2; lz = hz = 0; break;
	default: return -1;
	}
	const long long nt = (long long)s.bx * s.by;
	const long long ncol = (long long)std::max(0, nx - lx - hx) * std::max(0, ny - ly - hy);
	const int dz = std::max(0, ns - lz - hz);
	*ty = 1;
	if (lz == 0 && hz == 0) {
		*tx = (int)((ncol + nt * s.kc - 1) / (nt * s.kc));
		*tz = ncol > 0 ? 1 : 0;
	} else {
		*tx = (int)((ncol + nt - 1) / nt);
		*tz = (dz + s.kc - 1) / s.kc;
	}
	return 0;
}

}  // namespace kg

using namespace kg;

struct kg_batch_s {
	std::vector<kg_problem> probs;
	int dtype = KG_F32;
	int sms = 0;
	int shape = 0, ctas = 4;
	int total = 0;
	long long steps_done = 0;
	BatchDesc* d_desc = nullptr;   // device table for the current shape
	long long* d_step = nullptr;   // device step base
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	int graph_steps = 0;
};

static kg_status batch_build_table(kg_batch_s* b, int shape)
{
	std::vector<BatchDesc> h(b->probs.size());
	int first = 0;
	for (size_t q = 0; q < b->probs.size(); q++) {
		const kg_problem& p = b->probs[q];
		BatchDesc& d = h[q];
		memset(&d, 0, sizeof(d));
		d.stencil = p.stencil;
		d.nx = p.nx;
		d.ny = p.ny;
		d.ns = p.ns;
		for (int k = 0; k < 6; k++) d.c[k] = p.coef[k];
		if (p.stencil == KG_GAUSSBLUR)
			d.c[6] = 1. / (p.coef[0] + 4 * (p.coef[1] + p.coef[2] + p.coef[3] + p.coef[5]) + 8 * p.coef[4]);
		for (int k = 0; k < 4; k++) d.a[k] = p.arr[k];
		tiles_of(p.stencil, p.nx, p.ny, p.ns, k_shapes[shape], &d.tiles_x, &d.tiles_y, &d.tiles_z);
		d.first = first;
		const long long nt = (long long)d.tiles_x * d.tiles_y * d.tiles_z;
		if (first + nt > 0x7fffffffLL) return fail(KG_EINVAL, "kg_batch: more than 2^31 tiles");
		first += (int)nt;
	}
	cudaError_t e = cudaMemcpy(b->d_desc, h.data(), sizeof(BatchDesc) * h.size(), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return fail_cuda(e, "kg_batch: descriptor table");
	b->shape = shape;
	b->total = first;
	return KG_OK;
}

static cudaError_t batch_launch_steps(kg_batch_s* b, int nsteps, cudaStream_t st)
{
	const dim3 grid(b->sms * b->ctas);
	const int np = (int)b->probs.size();
	for (int s = 0; s < nsteps; s++) {
		cudaError_t e = (b->dtype == KG_F32)
			? launch_shape<FF, float>(b->shape, grid, b->d_desc, np, b->total, b->d_step, s, st)
			: launch_shape<SD, double>(b->shape, grid, b->d_desc, np, b->total, b->d_step, s, st);
		if (e != cudaSuccess) return e;
	}
	batch_advance<<<1, 32, 0, st>>>(b->d_step, nsteps);
	return cudaGetLastError();
}

static void drop_graph(kg_batch_s* b)
{
	if (b->exec) cudaGraphExecDestroy(b->exec);
	if (b->graph) cudaGraphDestroy(b->graph);
	b->exec = nullptr;
	b->graph = nullptr;
	b->graph_steps = 0;
}

static std::string batch_signature(const kg_batch_s* b)
{
	unsigned long long h = 1469598103934665603ULL;
	auto mix = [&](long long v) { h ^= (unsigned long long)v; h *= 1099511628211ULL; };
	mix(b->dtype);
	for (const kg_problem& p : b->probs) { mix(p.stencil); mix(p.nx); mix(p.ny); mix(p.ns); }
	cudaDeviceProp prop;
	int dev = 0;
	cudaGetDevice(&dev);
	cudaGetDeviceProperties(&prop, dev);
	char buf[512];
	snprintf(buf, sizeof(buf), "%s|sm%d|%zu|%016llx", prop.name, prop.multiProcessorCount, b->probs.size(), h);
	for (char* c = buf; *c; c++) if (*c == ' ') *c = '_';
	return buf;
}

extern "C" {

kg_status kg_batch_create(kg_batch* out, const kg_problem* probs, int nprob)
{
	clear_error();
	if (!out || !probs || nprob < 1 || nprob > kBatchMax)
		return fail(KG_EINVAL, "kg_batch_create: need 1..%d problems", kBatchMax);
	*out = nullptr;
	const int dt = probs[0].dtype;
	if (dt != KG_F32 && dt != KG_F64) return fail(KG_ENOTSUP, "kg_batch_create: batches are FP32 or FP64");
	for (int q = 0; q < nprob; q++) {
		const kg_problem& p = probs[q];
		if (p.dtype != dt) return fail(KG_EINVAL, "kg_batch_create: problem %d has another dtype", q);
		if (p.stencil != KG_LAPLACIAN && p.stencil != KG_DIVERGENCE && p.stencil != KG_WAVE13PT &&
			p.stencil != KG_GAUSSBLUR)
			return fail(KG_ENOTSUP, "kg_batch_create: problem %d: batches take laplacian, divergence, "
				"wave13pt and gaussblur", q);
		if (p.nx < 0 || p.ny < 0 || p.ns < 0 || (p.stencil == KG_GAUSSBLUR && p.ns != 1))
			return fail(KG_EINVAL, "kg_batch_create: problem %d: bad sizes", q);
		for (int k = 0; k < kg_stencil_narrays(p.stencil); k++)
			if (!p.arr[k]) return fail(KG_EINVAL, "kg_batch_create: problem %d: array %d is null", q, k);
	}
	kg_batch_s* b = new (std::nothrow) kg_batch_s();
	if (!b) return fail(KG_ENOMEM, "kg_batch_create");
	b->probs.assign(probs, probs + nprob);
	b->dtype = dt;
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
	if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_desc, sizeof(BatchDesc) * nprob);
	if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_step, sizeof(long long));
	if (e == cudaSuccess) e = cudaMemset(b->d_step, 0, sizeof(long long));
	kg_status s = fail_cuda(e, "kg_batch_create");
	if (s == KG_OK) s = batch_build_table(b, 0);
	if (s != KG_OK) {
		cudaFree(b->d_desc);
		cudaFree(b->d_step);
		delete b;
		return s;
	}
	*out = b;
	return KG_OK;
}

kg_status kg_batch_set_config(kg_batch b, int shape, int ctas_per_sm)
{
	clear_error();
	if (!b || shape < 0 || shape >= k_nshapes || ctas_per_sm < 1 || ctas_per_sm > 32)
		return fail(KG_EINVAL, "kg_batch_set_config: bad argument");
	drop_graph(b);
	b->ctas = ctas_per_sm;
	return batch_build_table(b, shape);
}

kg_status kg_batch_get_config(kg_batch b, kg_batch_config* cfg)
{
	clear_error();
	if (!b || !cfg) return fail(KG_EINVAL, "kg_batch_get_config: bad argument");
	cfg->shape = b->shape;
	cfg->bx = k_shapes[b->shape].bx;
	cfg->by = k_shapes[b->shape].by;
	cfg->kc = k_shapes[b->shape].kc;
	cfg->ctas_per_sm = b->ctas;
	cfg->tiles = b->total;
	cfg->nshapes = k_nshapes;
	cfg->steps_done = b->steps_done;
	return KG_OK;
}

kg_status kg_batch_step(kg_batch b, int nsteps, kg_stream_t stream)
{
	clear_error();
	if (!b || nsteps < 0) return fail(KG_EINVAL, "kg_batch_step: bad argument");
	if (nsteps == 0) return KG_OK;
	kg_status s = fail_cuda(batch_launch_steps(b, nsteps, (cudaStream_t)stream), "kg_batch_step");
	if (s == KG_OK) b->steps_done += nsteps;
	return s;
}

kg_status kg_batch_capture(kg_batch b, int nsteps)
{
	clear_error();
	if (!b || nsteps < 1) return fail(KG_EINVAL, "kg_batch_capture: bad argument");
	drop_graph(b);
	cudaStream_t cs;
	kg_status s = fail_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "kg_batch_capture");
	if (s != KG_OK) return s;
	s = fail_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "kg_batch_capture");
	if (s == KG_OK) {
		cudaError_t e = batch_launch_steps(b, nsteps, cs);
		cudaGraph_t g = nullptr;
		cudaError_t e2 = cudaStreamEndCapture(cs, &g);
		s = fail_cuda(e != cudaSuccess ? e : e2, "kg_batch_capture");
		if (s == KG_OK) {
			b->graph = g;
			s = fail_cuda(cudaGraphInstantiate(&b->exec, g, 0), "kg_batch_capture: instantiate");
		} else if (g) {
			cudaGraphDestroy(g);
		}
	}
	cudaStreamDestroy(cs);
	if (s != KG_OK) drop_graph(b);
	else b->graph_steps = nsteps;
	return s;
}

kg_status kg_batch_launch(kg_batch b, kg_stream_t stream)
{
	clear_error();
	if (!b || !b->exec) return fail(KG_EINVAL, "kg_batch_launch: no captured graph");
	kg_status s = fail_cuda(cudaGraphLaunch(b->exec, (cudaStream_t)stream), "kg_batch_launch");
	if (s == KG_OK) b->steps_done += b->graph_steps;
	return s;
}

kg_status kg_batch_tune(kg_batch b, const char* cache_path, kg_stream_t stream)
{
	clear_error();
	if (!b) return fail(KG_EINVAL, "kg_batch_tune: null batch");
	const std::string sig = batch_signature(b);
	if (cache_path) {
		FILE* f = fopen(cache_path, "r");
		if (f) {
			char key[256];
			int shape, ctas;
			while (fscanf(f, "%255s %d %d", key, &shape, &ctas) == 3) {
				if (sig == key && shape >= 0 && shape < k_nshapes && ctas >= 1 && ctas <= 32) {
					fclose(f);
					return kg_batch_set_config(b, shape, ctas);
				}
			}
			fclose(f);
		}
	}
	cudaStream_t st = (cudaStream_t)stream;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	float best = 1e30f;
	int best_shape = 0, best_ctas = 4;
	kg_status s = KG_OK;
	// Each trial advances the batch; the roles stay consistent because the
	// device step counter advances with them.
	for (int sh = 0; sh < k_nshapes && s == KG_OK; sh++) {
		// one wave of resident CTAs, one fewer per SM, half as many
		const int occ = b->dtype == KG_F32 ? shape_occupancy<FF, float>(sh) : shape_occupancy<SD, double>(sh);
		int cand[3] = {occ, occ > 1 ? occ - 1 : 1, occ > 1 ? occ / 2 : 1};
		for (int c = 0; c < 3 && s == KG_OK; c++) {
			if (c > 0 && (cand[c] == cand[c - 1] || (c == 2 && cand[2] == cand[0]))) continue;
			if ((s = kg_batch_set_config(b, sh, cand[c])) != KG_OK) break;
			if ((s = kg_batch_step(b, 1, stream)) != KG_OK) break;  // warm-up
			cudaEventRecord(e0, st);
			if ((s = kg_batch_step(b, 3, stream)) != KG_OK) break;
			cudaEventRecord(e1, st);
			if ((s = fail_cuda(cudaEventSynchronize(e1), "kg_batch_tune")) != KG_OK) break;
			float ms = 0;
			cudaEventElapsedTime(&ms, e0, e1);
			if (ms < best) { best = ms; best_shape = sh; best_ctas = cand[c]; }
		}
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if (s != KG_OK) return s;
	s = kg_batch_set_config(b, best_shape, best_ctas);
	if (s == KG_OK && cache_path) {
		FILE* f = fopen(cache_path, "a");
		if (f) {
			fprintf(f, "%s %d %d\n", sig.c_str(), best_shape, best_ctas);
			fclose(f);
		}
	}
	return s;
}

kg_status kg_batch_final_roles(kg_batch b, int q, kg_problem* out)
{
	clear_error();
	if (!b || !out || q < 0 || q >= (int)b->probs.size()) return fail(KG_EINVAL, "kg_batch_final_roles: bad argument");
	*out = b->probs[q];
	const long long s = b->steps_done;
	switch (out->stencil) {
	case KG_LAPLACIAN: case KG_GAUSSBLUR: {
		const int r = (int)(s & 1);
		out->arr[0] = b->probs[q].arr[r];
		out->arr[1] = b->probs[q].arr[r ^ 1];
		break;
	}
	case KG_WAVE13PT: {
		const int r = (int)(s % 3);
		for (int k = 0; k < 3; k++) out->arr[k] = b->probs[q].arr[(r + k) % 3];
		break;
	}
	default: break;
	}
	return KG_OK;
}

kg_status kg_batch_set_step(kg_batch b, long long step)
{
	clear_error();
	if (!b || step < 0) return fail(KG_EINVAL, "kg_batch_set_step: bad argument");
	kg_status s = fail_cuda(cudaMemcpy(b->d_step, &step, sizeof(step), cudaMemcpyHostToDevice), "kg_batch_set_step");
	if (s == KG_OK) b->steps_done = step;
	return s;
}

kg_status kg_batch_destroy(kg_batch b)
{
	clear_error();
	if (!b) return KG_OK;
	drop_graph(b);
	cudaFree(b->d_desc);
	cudaFree(b->d_step);
	delete b;
	return KG_OK;
}

}  // extern "C"
