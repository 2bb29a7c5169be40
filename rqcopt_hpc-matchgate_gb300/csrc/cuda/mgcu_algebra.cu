// FP64 algebra on the GPU: Riemannian projection of gradients and Hessians,
// retraction onto U(2)+U(2), and the truncated-CG trust-region subproblem.
#include "mgcu_common.cuh"

#include <vector>

namespace {

DevBuf g_u, g_eta, g_v, g_grad, g_hess, g_z, g_x, g_y, g_flag, g_dv, g_gv, g_H, g_vec;

// ---- projection (reference src/matchgate_target.c:901-967) ----
__global__ void k_project_grad(const mgg* __restrict__ v, const double* __restrict__ dg, int nb, double* __restrict__ grad, mgg* __restrict__ dvc)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= nb) return;
	mgg d;
	for (int q = 0; q < 4; q++)
	{
		d.c[q] = mgc_make(dg[i * 16 + 2 * q], dg[i * 16 + 2 * q + 1]);
		d.k[q] = mgc_make(dg[i * 16 + 8 + 2 * q], dg[i * 16 + 8 + 2 * q + 1]);
	}
	mgg_conj(&d);            // derivative convention
	dvc[i] = d;
	mgg_tangent_to_real(&v[i], &d, &grad[i * 8]);
}

// one thread per (i, j >= i, k): column k of block (i, j)
__global__ void k_project_hess(const mgg* __restrict__ v, const mgg* __restrict__ dvc, const double2* __restrict__ hess, int nb, double* __restrict__ H)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= nb * nb * 8) return;
	const int k = t % 8, ij = t / 8;
	const int i = ij / nb, j = ij % nb;
	if (j < i) return;
	const int m = 8 * nb;
	mgc h[64];
	for (int x = 0; x < 8; x++)
		for (int y = 0; y < 8; y++)
		{
			const double2 e = hess[(long)(i * 8 + x) * m + j * 8 + y];
			h[x * 8 + y] = mgc_make(e.x, e.y);
		}
	double r[8];
	mg_project_hessian_column(&v[i], &v[j], &dvc[i], i == j, h, k, r);
	for (int x = 0; x < 8; x++) H[(long)(i * 8 + x) * m + j * 8 + k] = r[x];
}

__global__ void k_mirror_real(int m, double* __restrict__ H)
{
	for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m * m; q += gridDim.x * blockDim.x)
	{
		const int r = q / m, c = q % m;
		if (c < r) H[(long)r * m + c] = H[(long)c * m + r];
	}
}

// ---- retraction (reference src/matchgate.c:548-562) ----
__global__ void k_retract(const mgg* __restrict__ u, const double* __restrict__ eta, int n, mgg* __restrict__ v)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) mgg_retract(&u[i], &eta[i * 8], &v[i]);
}

// ---- truncated CG (reference src/trust_region.c:17-146), one block ----
__device__ double block_dot(const double* a, const double* b, int n, double* red)
{
	double s = 0;
	for (int i = threadIdx.x; i < n; i += blockDim.x) s += a[i] * b[i];
	for (int m = 16; m > 0; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	__syncthreads();
	if (lane == 0) red[warp] = s;
	__syncthreads();
	double t = 0;
	for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
	__syncthreads();
	return t;
}

__device__ double boundary_step(const double* z, const double* d, int n, double radius, double* red)
{
	const double dd = block_dot(d, d, n, red);
	if (dd == 0) return 0;
	const double p = block_dot(z, d, n, red) / dd;
	const double q = (block_dot(z, z, n, red) - radius * radius) / dd;
	if (p == 0) return sqrt(-q);
	const double a = -(p + copysign(1.0, p) * sqrt(p * p - q));
	const double c = q / a;
	return a <= c ? c : a;
}

// work: r, d, hd (3n doubles); flag[0] = 1 when the step ended on the boundary
__global__ void __launch_bounds__(512) k_tcg(const double* __restrict__ grad, const double* __restrict__ hess, int n, double radius,
	int maxiter, double abstol, double reltol, double* __restrict__ z, double* __restrict__ work, int* __restrict__ flag)
{
	__shared__ double red[32];
	double* r = work;
	double* d = work + n;
	double* hd = work + 2 * n;
	for (int i = threadIdx.x; i < n; i += blockDim.x) { r[i] = grad[i]; z[i] = 0; d[i] = -grad[i]; }
	__syncthreads();
	double rsq = block_dot(r, r, n, red);
	const double stoptol = fmax(abstol, reltol * sqrt(rsq));
	int boundary = 0;
	for (int it = 0; it < maxiter; it++)
	{
		for (int i = threadIdx.x; i < n; i += blockDim.x)
		{
			double s = 0;
			const double* row = hess + (long)i * n;
			for (int j = 0; j < n; j++) s += row[j] * d[j];
			hd[i] = s;
		}
		__syncthreads();
		const double dhd = block_dot(d, hd, n, red);
		const double tb = boundary_step(z, d, n, radius, red);
		const double alpha = rsq / dhd;
		if (dhd <= 0 || alpha > tb)
		{
			for (int i = threadIdx.x; i < n; i += blockDim.x) z[i] += tb * d[i];
			boundary = 1;
			break;
		}
		for (int i = threadIdx.x; i < n; i += blockDim.x) { r[i] += alpha * hd[i]; z[i] += alpha * d[i]; }
		__syncthreads();
		const double rsq1 = block_dot(r, r, n, red);
		if (sqrt(rsq1) <= stoptol) break;
		const double beta = rsq1 / rsq;
		for (int i = threadIdx.x; i < n; i += blockDim.x) d[i] = beta * d[i] - r[i];
		__syncthreads();
		rsq = rsq1;
	}
	if (threadIdx.x == 0) flag[0] = boundary;
}

__global__ void k_matvec(const double* __restrict__ H, const double* __restrict__ x, int n, double* __restrict__ y)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		double s = 0;
		for (int j = 0; j < n; j++) s += H[(long)i * n + j] * x[j];
		y[i] = s;
	}
}

__global__ void k_dense_matvec(const double2* __restrict__ U, long n, const double2* __restrict__ x, double2* __restrict__ y)
{
	for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
	{
		double sr = 0, si = 0;
		for (long j = 0; j < n; j++)
		{
			const double2 a = U[i * n + j], b = x[j];
			sr += a.x * b.x - a.y * b.y;
			si += a.x * b.y + a.y * b.x;
		}
		y[i] = make_double2(sr, si);
	}
}

#define TRY(x) do { int _r = (x); if (_r) return _r; } while (0)

int up(DevBuf& b, const void* h, size_t n) { TRY(b.alloc(n)); MGCU_TRY(cudaMemcpyAsync(b.p, h, n, cudaMemcpyHostToDevice, mgcu_stream())); return 0; }
int down(void* h, const DevBuf& b, size_t n) { MGCU_TRY(cudaMemcpyAsync(h, b.p, n, cudaMemcpyDeviceToHost, mgcu_stream())); return 0; }
int sync() { MGCU_TRY(cudaStreamSynchronize(mgcu_stream())); return 0; }

}  // namespace

int mgcu_project_dev(const mgg* vblocks, int nb, const double* dgrad_dev, const double* hess_dev, double* grad_vec, double* H)
{
	MgcuContext* c = mgcu_ctx();
	if (!c) return MG_ERR_DEVICE;
	const int m = 8 * nb;
	TRY(up(g_v, vblocks, sizeof(mgg) * nb));
	TRY(g_dv.alloc(sizeof(mgg) * nb));
	TRY(g_gv.alloc(sizeof(double) * m));
	k_project_grad<<<(nb + 63) / 64, 64, 0, mgcu_stream()>>>(g_v.as<mgg>(), dgrad_dev, nb, g_gv.as<double>(), g_dv.as<mgg>());
	MGCU_LAUNCHED();
	if (grad_vec) TRY(down(grad_vec, g_gv, sizeof(double) * m));
	if (hess_dev && H)
	{
		TRY(g_H.alloc(sizeof(double) * m * m));
		k_project_hess<<<(nb * nb * 8 + 63) / 64, 64, 0, mgcu_stream()>>>(g_v.as<mgg>(), g_dv.as<mgg>(), (const double2*)hess_dev, nb, g_H.as<double>());
		MGCU_LAUNCHED();
		k_mirror_real<<<(m * m + 255) / 256, 256, 0, mgcu_stream()>>>(m, g_H.as<double>());
		MGCU_LAUNCHED();
		TRY(down(H, g_H, sizeof(double) * m * m));
	}
	return sync();
}

extern "C" int mgcu_retract(const mgg* u, const double* eta, int n, mgg* v)
{
	MgcuContext* c = mgcu_ctx();
	if (!c) return MG_ERR_DEVICE;
	TRY(up(g_u, u, sizeof(mgg) * n));
	TRY(up(g_eta, eta, sizeof(double) * 8 * n));
	TRY(g_v.alloc(sizeof(mgg) * n));
	k_retract<<<(n + 63) / 64, 64, 0, mgcu_stream()>>>(g_u.as<mgg>(), g_eta.as<double>(), n, g_v.as<mgg>());
	MGCU_LAUNCHED();
	TRY(down(v, g_v, sizeof(mgg) * n));
	return sync();
}

extern "C" int mgcu_truncated_cg(const double* grad, const double* hess, int n, double radius, int maxiter, double abstol, double reltol, double* z)
{
	MgcuContext* c = mgcu_ctx();
	if (!c) return MG_ERR_DEVICE;
	TRY(up(g_grad, grad, sizeof(double) * n));
	TRY(up(g_hess, hess, sizeof(double) * n * n));
	TRY(g_z.alloc(sizeof(double) * n));
	TRY(g_x.alloc(sizeof(double) * 3 * n));
	TRY(g_flag.alloc(sizeof(int)));
	k_tcg<<<1, 512, 0, mgcu_stream()>>>(g_grad.as<double>(), g_hess.as<double>(), n, radius, maxiter, abstol, reltol, g_z.as<double>(), g_x.as<double>(), g_flag.as<int>());
	MGCU_LAUNCHED();
	int flag = 0;
	TRY(down(z, g_z, sizeof(double) * n));
	TRY(down(&flag, g_flag, sizeof(int)));
	TRY(sync());
	return flag;
}

extern "C" int mgcu_matvec(const double* H, const double* x, int n, double* y)
{
	MgcuContext* c = mgcu_ctx();
	if (!c) return MG_ERR_DEVICE;
	TRY(up(g_hess, H, sizeof(double) * n * n));
	TRY(up(g_x, x, sizeof(double) * n));
	TRY(g_y.alloc(sizeof(double) * n));
	k_matvec<<<(n + 127) / 128, 128, 0, mgcu_stream()>>>(g_hess.as<double>(), g_x.as<double>(), n, g_y.as<double>());
	MGCU_LAUNCHED();
	TRY(down(y, g_y, sizeof(double) * n));
	return sync();
}

extern "C" int mgcu_dense_matvec(const void* U, int L, const mgc* psi, mgc* out)
{
	MgcuContext* c = mgcu_ctx();
	if (!c) return MG_ERR_DEVICE;
	const long n = 1L << L;
	TRY(up(g_x, psi, sizeof(double2) * n));
	TRY(g_y.alloc(sizeof(double2) * n));
	k_dense_matvec<<<(int)((n + 127) / 128), 128, 0, mgcu_stream()>>>((const double2*)U, n, g_x.as<double2>(), g_y.as<double2>());
	MGCU_LAUNCHED();
	TRY(down(out, g_y, sizeof(double2) * n));
	return sync();
}

