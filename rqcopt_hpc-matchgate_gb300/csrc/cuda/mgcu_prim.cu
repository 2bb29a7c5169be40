// Per-vector primitives in FP64 on full 2^L state vectors: one gate per launch,
// used by the single-vector API (gate.h, quantum_circuit.h, matchgate_brickwall.h).
// The batched evaluations use the parity-sector engine in mgcu_engine.cu instead.
//
// Index convention (reference src/gate.c:581-652): qubit 0 is the most significant
// bit; for a gate on wires (i, j) the local index is 2*bit_i + bit_j, so the
// quartet of a base index a (bits i, j clear) is x = a, y = a|bj, z = a|bi,
// w = a|bi|bj.  The corner block maps (x, w), the center block maps (y, z).
#include "mgcu_common.cuh"

namespace {

struct GateD { double2 c[4]; double2 k[4]; };

__device__ __forceinline__ long ins0(long t, int p) { return ((t >> p) << (p + 1)) | (t & ((1L << p) - 1)); }
__device__ __forceinline__ long qbase(long t, int pa, int pb)
{
	const int lo = pa < pb ? pa : pb, hi = pa < pb ? pb : pa;
	return ins0(ins0(t, lo), hi);
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cmad2(double2 a, double2 x, double2 b, double2 y) { return cadd(cmul(a, x), cmul(b, y)); }

__global__ void k_apply(GateD g, int pi, int pj, int L, int ns, const double2* __restrict__ in, double2* __restrict__ out)
{
	const long nq = 1L << (L - 2);
	const long bi = 1L << pi, bj = 1L << pj;
	for (long u = blockIdx.x * (long)blockDim.x + threadIdx.x; u < nq * ns; u += (long)gridDim.x * blockDim.x)
	{
		const long t = u / ns;
		const int s = (int)(u - t * ns);
		const long a = qbase(t, pi, pj);
		const double2 x = in[a * ns + s], y = in[(a | bj) * ns + s], z = in[(a | bi) * ns + s], w = in[(a | bi | bj) * ns + s];
		out[a * ns + s]             = cmad2(g.k[0], x, g.k[1], w);
		out[(a | bj) * ns + s]      = cmad2(g.c[0], y, g.c[1], z);
		out[(a | bi) * ns + s]      = cmad2(g.c[2], y, g.c[3], z);
		out[(a | bi | bj) * ns + s] = cmad2(g.k[2], x, g.k[3], w);
	}
}

// 8 complex gradient entries (center 0..3, corner 4..7) reduced over the block and
// written to part[blockIdx.x*8 ...]; dpsi = G^T dpsi_out
__global__ void __launch_bounds__(256) k_backward(GateD g, int pi, int pj, int L, const double2* __restrict__ psi,
	const double2* __restrict__ dout, double2* __restrict__ dpsi, double2* __restrict__ part)
{
	const long nq = 1L << (L - 2);
	const long bi = 1L << pi, bj = 1L << pj;
	double2 acc[8];
	for (int e = 0; e < 8; e++) acc[e] = make_double2(0, 0);
	for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nq; t += (long)gridDim.x * blockDim.x)
	{
		const long a = qbase(t, pi, pj);
		const double2 x = psi[a], y = psi[a | bj], z = psi[a | bi], w = psi[a | bi | bj];
		const double2 dx = dout[a], dy = dout[a | bj], dz = dout[a | bi], dw = dout[a | bi | bj];
		acc[0] = cadd(acc[0], cmul(dy, y)); acc[1] = cadd(acc[1], cmul(dy, z));
		acc[2] = cadd(acc[2], cmul(dz, y)); acc[3] = cadd(acc[3], cmul(dz, z));
		acc[4] = cadd(acc[4], cmul(dx, x)); acc[5] = cadd(acc[5], cmul(dx, w));
		acc[6] = cadd(acc[6], cmul(dw, x)); acc[7] = cadd(acc[7], cmul(dw, w));
		if (dpsi)
		{
			dpsi[a]           = cmad2(g.k[0], dx, g.k[2], dw);
			dpsi[a | bj]      = cmad2(g.c[0], dy, g.c[2], dz);
			dpsi[a | bi]      = cmad2(g.c[1], dy, g.c[3], dz);
			dpsi[a | bi | bj] = cmad2(g.k[1], dx, g.k[3], dw);
		}
	}
	__shared__ double2 red[8][256];
	for (int e = 0; e < 8; e++) red[e][threadIdx.x] = acc[e];
	__syncthreads();
	for (int s = blockDim.x / 2; s > 0; s >>= 1)
	{
		if (threadIdx.x < s)
			for (int e = 0; e < 8; e++) red[e][threadIdx.x] = cadd(red[e][threadIdx.x], red[e][threadIdx.x + s]);
		__syncthreads();
	}
	if (threadIdx.x < 8) part[blockIdx.x * 8 + threadIdx.x] = red[threadIdx.x][0];
}

// per-state gradients of an interleaved array against one upstream derivative:
// part[(blockIdx.x * ns + s) * 8 + e]
__global__ void __launch_bounds__(128) k_backward_array(int pi, int pj, int L, int ns, const double2* __restrict__ psi,
	const double2* __restrict__ dout, double2* __restrict__ part)
{
	const long nq = 1L << (L - 2);
	const long bi = 1L << pi, bj = 1L << pj;
	const int s = blockIdx.y;
	double2 acc[8];
	for (int e = 0; e < 8; e++) acc[e] = make_double2(0, 0);
	for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nq; t += (long)gridDim.x * blockDim.x)
	{
		const long a = qbase(t, pi, pj);
		const double2 x = psi[a * ns + s], y = psi[(a | bj) * ns + s], z = psi[(a | bi) * ns + s], w = psi[(a | bi | bj) * ns + s];
		const double2 dx = dout[a], dy = dout[a | bj], dz = dout[a | bi], dw = dout[a | bi | bj];
		acc[0] = cadd(acc[0], cmul(dy, y)); acc[1] = cadd(acc[1], cmul(dy, z));
		acc[2] = cadd(acc[2], cmul(dz, y)); acc[3] = cadd(acc[3], cmul(dz, z));
		acc[4] = cadd(acc[4], cmul(dx, x)); acc[5] = cadd(acc[5], cmul(dx, w));
		acc[6] = cadd(acc[6], cmul(dw, x)); acc[7] = cadd(acc[7], cmul(dw, w));
	}
	__shared__ double2 red[8][128];
	for (int e = 0; e < 8; e++) red[e][threadIdx.x] = acc[e];
	__syncthreads();
	for (int h = blockDim.x / 2; h > 0; h >>= 1)
	{
		if (threadIdx.x < h)
			for (int e = 0; e < 8; e++) red[e][threadIdx.x] = cadd(red[e][threadIdx.x], red[e][threadIdx.x + h]);
		__syncthreads();
	}
	if (threadIdx.x < 8) part[((long)blockIdx.x * ns + s) * 8 + threadIdx.x] = red[threadIdx.x][0];
}

// sum partials in block order: out[r] = sum_b part[b * nrow + r]
__global__ void k_sum_partials(const double2* __restrict__ part, int nblk, int nrow, double2* __restrict__ out)
{
	for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrow; r += gridDim.x * blockDim.x)
	{
		double2 s = make_double2(0, 0);
		for (int b = 0; b < nblk; b++) s = cadd(s, part[(long)b * nrow + r]);
		out[r] = s;
	}
}

// 8 placeholder states (src/gate.c:982-1057) or 16 for a general 4x4 gate (src/gate.c:1066-1141)
__global__ void k_placeholder(int pi, int pj, int L, int nout, const double2* __restrict__ psi, double2* __restrict__ out)
{
	const long nq = 1L << (L - 2);
	const long bi = 1L << pi, bj = 1L << pj;
	for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nq; t += (long)gridDim.x * blockDim.x)
	{
		const long a = qbase(t, pi, pj);
		const long idx[4] = { a, a | bj, a | bi, a | bi | bj };
		const double2 v[4] = { psi[idx[0]], psi[idx[1]], psi[idx[2]], psi[idx[3]] };
		const double2 zero = make_double2(0, 0);
		for (int r = 0; r < 4; r++)
			for (int e = 0; e < nout; e++) out[idx[r] * nout + e] = zero;
		if (nout == 8)
		{
			out[idx[1] * 8 + 0] = v[1]; out[idx[1] * 8 + 1] = v[2];
			out[idx[2] * 8 + 2] = v[1]; out[idx[2] * 8 + 3] = v[2];
			out[idx[0] * 8 + 4] = v[0]; out[idx[0] * 8 + 5] = v[3];
			out[idx[3] * 8 + 6] = v[0]; out[idx[3] * 8 + 7] = v[3];
		}
		else
		{
			// entry (r, s) of the 4x4 gate in the local order 2*bit_i + bit_j: out|r> = psi|s>
			for (int r = 0; r < 4; r++)
				for (int s = 0; s < 4; s++) out[idx[r] * 16 + r * 4 + s] = v[s];
		}
	}
}

GateD to_gate(const mgg* g)
{
	GateD d;
	for (int q = 0; q < 4; q++)
	{
		d.c[q] = make_double2(g->c[q].re, g->c[q].im);
		d.k[q] = make_double2(g->k[q].re, g->k[q].im);
	}
	return d;
}

int grid_for(long work, int threads)
{
	MgcuContext* c = mgcu_ctx();
	long b = (work + threads - 1) / threads;
	const long cap = (long)c->nsm * 16;
	if (b > cap) b = cap;
	return (int)(b < 1 ? 1 : b);
}

// growable scratch buffers for the single-vector API (callers hold the library lock)
DevBuf g_a, g_b, g_c, g_d, g_part, g_out;

// ---- single-vector sweeps on device buffers ----
int dev_apply(const mgg* g, int i, int j, int L, int ns, const double2* in, double2* out)
{
	MgcuContext* c = mgcu_ctx();
	const long nq = 1L << (L - 2);
	k_apply<<<grid_for(nq * ns, 256), 256, 0, mgcu_stream()>>>(to_gate(g), L - 1 - i, L - 1 - j, L, ns, in, out);
	MGCU_LAUNCHED();
	return 0;
}

int dev_backward(const mgg* g, int i, int j, int L, const double2* psi, const double2* dout, double2* dpsi, double2* dg_dev)
{
	MgcuContext* c = mgcu_ctx();
	const long nq = 1L << (L - 2);
	const int nb = grid_for(nq, 256);
	int e = g_part.alloc(sizeof(double2) * 8 * nb);
	if (e) return e;
	k_backward<<<nb, 256, 0, mgcu_stream()>>>(to_gate(g), L - 1 - i, L - 1 - j, L, psi, dout, dpsi, g_part.as<double2>());
	MGCU_LAUNCHED();
	k_sum_partials<<<1, 32, 0, mgcu_stream()>>>(g_part.as<double2>(), nb, 8, dg_dev);
	MGCU_LAUNCHED();
	return 0;
}

int dev_backward_array(int i, int j, int L, int ns, const double2* psi, const double2* dout, double2* dg_dev)
{
	MgcuContext* c = mgcu_ctx();
	const long nq = 1L << (L - 2);
	int nb = grid_for(nq, 128);
	if (nb > 64) nb = 64;
	int e = g_part.alloc(sizeof(double2) * 8 * ns * nb);
	if (e) return e;
	k_backward_array<<<dim3(nb, ns), 128, 0, mgcu_stream()>>>(L - 1 - i, L - 1 - j, L, ns, psi, dout, g_part.as<double2>());
	MGCU_LAUNCHED();
	k_sum_partials<<<1, 128, 0, mgcu_stream()>>>(g_part.as<double2>(), nb, 8 * ns, dg_dev);
	MGCU_LAUNCHED();
	return 0;
}

int dev_placeholder(int i, int j, int L, int nout, const double2* psi, double2* out)
{
	MgcuContext* c = mgcu_ctx();
	const long nq = 1L << (L - 2);
	k_placeholder<<<grid_for(nq, 128), 128, 0, mgcu_stream()>>>(L - 1 - i, L - 1 - j, L, nout, psi, out);
	MGCU_LAUNCHED();
	return 0;
}

int sync_stream()
{
	MGCU_TRY(cudaStreamSynchronize(mgcu_stream()));
	return 0;
}

int h2d(void* dst, const void* src, size_t n) { MGCU_TRY(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, mgcu_stream())); return 0; }
int d2h(void* dst, const void* src, size_t n) { MGCU_TRY(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, mgcu_stream())); return 0; }

void gate_from_dev(const double2* d, mgg* g)
{
	for (int q = 0; q < 4; q++) { g->c[q] = mgc_make(d[q].x, d[q].y); g->k[q] = mgc_make(d[q + 4].x, d[q + 4].y); }
}

}  // namespace

#define CTX_OR_FAIL() do { if (!mgcu_ctx()) return MG_ERR_DEVICE; } while (0)
#define TRY(x) do { int _r = (x); if (_r) return _r; } while (0)

extern "C" int mgcu_prim_apply(const mgg* g, int i, int j, int L, int ns, const mgc* psi, mgc* out)
{
	CTX_OR_FAIL();
	const size_t bytes = sizeof(double2) * ns * ((size_t)1 << L);
	TRY(g_a.alloc(bytes)); TRY(g_b.alloc(bytes));
	TRY(h2d(g_a.p, psi, bytes));
	TRY(dev_apply(g, i, j, L, ns, g_a.as<double2>(), g_b.as<double2>()));
	TRY(d2h(out, g_b.p, bytes));
	return sync_stream();
}

extern "C" int mgcu_prim_backward(const mgg* g, int i, int j, int L, const mgc* psi, const mgc* dpsi_out, mgc* dpsi, mgg* dg)
{
	CTX_OR_FAIL();
	const size_t bytes = sizeof(double2) * ((size_t)1 << L);
	TRY(g_a.alloc(bytes)); TRY(g_b.alloc(bytes)); TRY(g_c.alloc(bytes)); TRY(g_out.alloc(sizeof(double2) * 8));
	TRY(h2d(g_a.p, psi, bytes)); TRY(h2d(g_b.p, dpsi_out, bytes));
	TRY(dev_backward(g, i, j, L, g_a.as<double2>(), g_b.as<double2>(), g_c.as<double2>(), g_out.as<double2>()));
	double2 h[8];
	TRY(d2h(dpsi, g_c.p, bytes));
	TRY(d2h(h, g_out.p, sizeof(h)));
	TRY(sync_stream());
	gate_from_dev(h, dg);
	return 0;
}

extern "C" int mgcu_prim_backward_array(const mgg* g, int i, int j, int L, int ns, const mgc* psi, const mgc* dpsi_out, mgg* dgs)
{
	(void)g;
	CTX_OR_FAIL();
	const size_t n = (size_t)1 << L;
	TRY(g_a.alloc(sizeof(double2) * n * ns)); TRY(g_b.alloc(sizeof(double2) * n)); TRY(g_out.alloc(sizeof(double2) * 8 * ns));
	TRY(h2d(g_a.p, psi, sizeof(double2) * n * ns)); TRY(h2d(g_b.p, dpsi_out, sizeof(double2) * n));
	TRY(dev_backward_array(i, j, L, ns, g_a.as<double2>(), g_b.as<double2>(), g_out.as<double2>()));
	double2* h = (double2*)malloc(sizeof(double2) * 8 * ns);
	if (!h) return MG_ERR_ALLOC;
	int r = d2h(h, g_out.p, sizeof(double2) * 8 * ns);
	if (!r) r = sync_stream();
	if (!r) for (int s = 0; s < ns; s++) gate_from_dev(h + 8 * s, &dgs[s]);
	free(h);
	return r;
}

extern "C" int mgcu_prim_placeholder(int i, int j, int L, int nout, const mgc* psi, mgc* out)
{
	CTX_OR_FAIL();
	const size_t n = (size_t)1 << L;
	TRY(g_a.alloc(sizeof(double2) * n)); TRY(g_b.alloc(sizeof(double2) * n * nout));
	TRY(h2d(g_a.p, psi, sizeof(double2) * n));
	TRY(dev_placeholder(i, j, L, nout, g_a.as<double2>(), g_b.as<double2>()));
	TRY(d2h(out, g_b.p, sizeof(double2) * n * nout));
	return sync_stream();
}

// forward sweep keeping every gate's input (reference src/quantum_circuit.c:90-108)
extern "C" int mgcu_circuit_forward(const mgg* gates, const int* wires, int ngates, int L, const mgc* psi, mgc* cache, mgc* out)
{
	CTX_OR_FAIL();
	const size_t n = (size_t)1 << L, bytes = sizeof(double2) * n;
	// device cache: slot g holds the input of gate g, slot ngates the output
	TRY(g_c.alloc(bytes * (ngates + 1)));
	double2* d = g_c.as<double2>();
	TRY(h2d(d, psi, bytes));
	for (int g = 0; g < ngates; g++) TRY(dev_apply(&gates[g], wires[2 * g], wires[2 * g + 1], L, 1, d + g * n, d + (g + 1) * n));
	if (cache && ngates > 0) TRY(d2h(cache, d, bytes * ngates));
	TRY(d2h(out, d + (size_t)ngates * n, bytes));
	return sync_stream();
}

// backward sweep (reference src/quantum_circuit.c:115-140)
extern "C" int mgcu_circuit_backward(const mgg* gates, const int* wires, int ngates, int L, const mgc* cache, const mgc* dpsi_out,
	mgc* dpsi, mgg* dgates)
{
	CTX_OR_FAIL();
	const size_t n = (size_t)1 << L, bytes = sizeof(double2) * n;
	TRY(g_c.alloc(bytes * (ngates > 0 ? ngates : 1)));
	TRY(g_a.alloc(bytes)); TRY(g_b.alloc(bytes)); TRY(g_out.alloc(sizeof(double2) * 8 * (ngates > 0 ? ngates : 1)));
	double2* cd = g_c.as<double2>();
	if (ngates > 0) TRY(h2d(cd, cache, bytes * ngates));
	TRY(h2d(g_a.p, dpsi_out, bytes));
	double2* cur = g_a.as<double2>();
	double2* nxt = g_b.as<double2>();
	for (int g = ngates - 1; g >= 0; g--)
	{
		TRY(dev_backward(&gates[g], wires[2 * g], wires[2 * g + 1], L, cd + g * n, cur, nxt, g_out.as<double2>() + 8 * g));
		double2* s = cur; cur = nxt; nxt = s;
	}
	TRY(d2h(dpsi, cur, bytes));
	double2* h = (double2*)malloc(sizeof(double2) * 8 * (ngates > 0 ? ngates : 1));
	if (!h) return MG_ERR_ALLOC;
	int r = d2h(h, g_out.p, sizeof(double2) * 8 * ngates);
	if (!r) r = sync_stream();
	if (!r) for (int g = 0; g < ngates; g++) gate_from_dev(h + 8 * g, &dgates[g]);
	free(h);
	return r;
}

// per-column Hessian sweep (reference src/matchgate_brickwall.c:137-260, :308-435)
namespace {
__global__ void k_hess_accumulate(const double2* __restrict__ h, int nlayers, int bi, int bj, double mult, double2* __restrict__ hess)
{
	// h: [8 states x][8 entries y(center 0..3, corner 4..7)]
	const int t = threadIdx.x;
	if (t < 64)
	{
		const int x = t / 8, y = t % 8;
		const long idx = ((long)(bi * 8 + x) * nlayers + bj) * 8 + y;
		const double2 v = h[x * 8 + y];
		hess[idx].x += mult * v.x;
		hess[idx].y += mult * v.y;
	}
}

__global__ void k_hess_symmetrize(int nb, double2* __restrict__ hess)
{
	// diagonal blocks: A + A^T ; lower blocks: mirror of the upper ones
	const int m = nb * 8;
	for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m * m; q += gridDim.x * blockDim.x)
	{
		const int r = q / m, c = q % m;
		const int bi = r / 8, bj = c / 8;
		if (bi == bj && (c % 8) < (r % 8))
		{
			const long p1 = (long)r * m + c, p2 = (long)c * m + r;
			const double2 s = cadd(hess[p1], hess[p2]);
			hess[p1] = s; hess[p2] = s;
		}
		else if (bi == bj && (c % 8) == (r % 8))
		{
			hess[(long)r * m + c].x *= 2; hess[(long)r * m + c].y *= 2;
		}
	}
}

__global__ void k_hess_mirror(int nb, double2* __restrict__ hess)
{
	const int m = nb * 8;
	for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m * m; q += gridDim.x * blockDim.x)
	{
		const int r = q / m, c = q % m;
		if (c / 8 < r / 8) hess[(long)r * m + c] = hess[(long)c * m + r];
	}
}
}  // namespace

extern "C" int mgcu_brickwall_backward_hessian(const mgg* vlist, int nlayers, const int* perms, int L, int ti, const mgc* cache,
	const mgc* dpsi_out, mgc* dpsi, mgg* dvlist, mgc* hess)
{
	CTX_OR_FAIL();
	MgcuContext* c = mgcu_ctx();
	const int half = L / 2, ng = nlayers * half;
	const size_t n = (size_t)1 << L, bytes = sizeof(double2) * n;
	DevBuf dcache, gcache, t0, t1, hdev, hblk, dgd;
	TRY(dcache.alloc(bytes * ng)); TRY(gcache.alloc(bytes * ng));
	TRY(t0.alloc(bytes * 8)); TRY(t1.alloc(bytes * 8));
	TRY(hdev.alloc(sizeof(double2) * 64 * nlayers * nlayers)); TRY(hblk.alloc(sizeof(double2) * 64)); TRY(dgd.alloc(sizeof(double2) * 8 * ng));
	double2* C = dcache.as<double2>();
	double2* G = gcache.as<double2>();
	TRY(h2d(C, cache, bytes * ng));
	TRY(h2d(G + (size_t)(ng - 1) * n, dpsi_out, bytes));
	TRY(g_a.alloc(bytes));
	// gradient, keeping the derivative entering each gate's backward step
	int k = ng - 1;
	for (int l = nlayers - 1; l >= 0; l--)
		for (int p = L - 2; p >= 0; p -= 2)
		{
			double2* dst = (k > 0) ? G + (size_t)(k - 1) * n : g_a.as<double2>();
			TRY(dev_backward(&vlist[l], perms[l * L + p], perms[l * L + p + 1], L, C + (size_t)k * n, G + (size_t)k * n, dst, dgd.as<double2>() + 8 * k));
			k--;
		}
	MGCU_TRY(cudaMemsetAsync(hdev.p, 0, sizeof(double2) * 64 * nlayers * nlayers, mgcu_stream()));
	double2* cur = t0.as<double2>();
	double2* nxt = t1.as<double2>();
	for (int i = 0; i < nlayers; i++)
	{
		const int rmax = ti ? 1 : half;
		for (int rr = 0; rr < rmax; rr++)
		{
			const int r = 2 * rr;
			const int kp = i * half + rr;
			cur = t0.as<double2>(); nxt = t1.as<double2>();
			TRY(dev_placeholder(perms[i * L + r], perms[i * L + r + 1], L, 8, C + (size_t)kp * n, cur));
			int lidx = kp + 1;
			for (int j = i; j < nlayers; j++)
			{
				int o = 1;
				for (int s = 0; s < L; s += 2)
				{
					if (j == i && s <= r) continue;
					double mult = 1.0;
					if (ti) { mult = half; if (j == i) mult -= o; }
					o++;
					TRY(dev_backward_array(perms[j * L + s], perms[j * L + s + 1], L, 8, cur, G + (size_t)lidx * n, hblk.as<double2>()));
					k_hess_accumulate<<<1, 64, 0, mgcu_stream()>>>(hblk.as<double2>(), nlayers, i, j, mult, hdev.as<double2>());
					MGCU_LAUNCHED();
					if (j < nlayers - 1 || s < L - 2)
					{
						TRY(dev_apply(&vlist[j], perms[j * L + s], perms[j * L + s + 1], L, 8, cur, nxt));
						double2* sw = cur; cur = nxt; nxt = sw;
					}
					lidx++;
				}
			}
		}
	}
	k_hess_symmetrize<<<grid_for((long)64 * nlayers * nlayers, 256), 256, 0, mgcu_stream()>>>(nlayers, hdev.as<double2>());
	MGCU_LAUNCHED();
	k_hess_mirror<<<grid_for((long)64 * nlayers * nlayers, 256), 256, 0, mgcu_stream()>>>(nlayers, hdev.as<double2>());
	MGCU_LAUNCHED();
	TRY(d2h(dpsi, g_a.p, bytes));
	TRY(d2h(hess, hdev.p, sizeof(double2) * 64 * nlayers * nlayers));
	double2* dg = (double2*)malloc(sizeof(double2) * 8 * ng);
	if (!dg) return MG_ERR_ALLOC;
	int rc = d2h(dg, dgd.p, sizeof(double2) * 8 * ng);
	if (!rc) rc = sync_stream();
	if (!rc)
	{
		// per-layer sums in the reference's order (last pair first)
		k = ng - 1;
		for (int l = nlayers - 1; l >= 0; l--)
		{
			mgg_zero(&dvlist[l]);
			for (int p = L - 2; p >= 0; p -= 2)
			{
				mgg t;
				gate_from_dev(dg + 8 * k, &t);
				mgg_add(&dvlist[l], &t);
				k--;
			}
		}
	}
	free(dg);
	return rc;
}
