// Device context, error reporting, launch counting, and the peak-rate
// microkernels used as roofline denominators.
#include "mgcu_common.cuh"

#include <atomic>
#include <stdlib.h>

static MgcuContext g_ctx;
static int g_ctx_state = 0;   // 0 uninitialised, 1 ready, -1 failed
static std::atomic<long> g_launches(0);

int mgcu_check(cudaError_t e, const char* what, const char* file, int line)
{
	mg_set_error("CUDA error in %s (%s:%d): %s", what, file, line, cudaGetErrorString(e));
	return (e == cudaErrorMemoryAllocation) ? MG_ERR_ALLOC : MG_ERR_DEVICE;
}

MgcuContext* mgcu_ctx()
{
	if (g_ctx_state == 1) return &g_ctx;
	if (g_ctx_state == -1) return nullptr;
	int ndev = 0;
	cudaError_t e = cudaGetDeviceCount(&ndev);
	if (e != cudaSuccess || ndev == 0)
	{
		mg_set_error("no CUDA device available (%s); this library has no CPU path", e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
		g_ctx_state = -1;
		return nullptr;
	}
	// MG_DEVICE selects the GPU (one process per GPU; default 0)
	const char* env = getenv("MG_DEVICE");
	g_ctx.device = env ? atoi(env) : 0;
	cudaDeviceProp prop;
	if (g_ctx.device < 0 || g_ctx.device >= ndev || cudaSetDevice(g_ctx.device) != cudaSuccess ||
		cudaGetDeviceProperties(&prop, g_ctx.device) != cudaSuccess)
	{
		mg_set_error("cannot open CUDA device %d (of %d)", g_ctx.device, ndev);
		g_ctx_state = -1;
		return nullptr;
	}
	g_ctx.nsm = prop.multiProcessorCount;
	g_ctx.smem_optin = prop.sharedMemPerBlockOptin;
	if (cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking) != cudaSuccess ||
		cudaEventCreate(&g_ctx.ev0) != cudaSuccess || cudaEventCreate(&g_ctx.ev1) != cudaSuccess)
	{
		mg_set_error("cannot create the CUDA stream of the matchgate library");
		g_ctx_state = -1;
		return nullptr;
	}
	g_ctx_state = 1;
	return &g_ctx;
}

// the stream this host thread issues its work on: the library's stream, or one the thread
// selected (mgcu_stream_set), so that two host threads can keep work in flight on the GPU
// at the same time (each waits for its own stream outside the library lock)
static thread_local cudaStream_t t_stream = nullptr;

cudaStream_t mgcu_stream()
{
	if (t_stream) return t_stream;
	MgcuContext* c = mgcu_ctx();
	return c ? c->stream : nullptr;
}

extern "C" void* mgcu_stream_create(void)
{
	if (!mgcu_ctx()) return nullptr;
	cudaStream_t s = nullptr;
	if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { mg_set_error("cannot create a CUDA stream"); return nullptr; }
	return (void*)s;
}

extern "C" void mgcu_stream_set(void* s) { t_stream = (cudaStream_t)s; }

extern "C" int mgcu_stream_sync(void)
{
	cudaStream_t s = mgcu_stream();
	if (!s) return MG_ERR_DEVICE;
	MGCU_TRY(cudaStreamSynchronize(s));
	return 0;
}

extern "C" void mgcu_stream_destroy(void* s)
{
	if (s) cudaStreamDestroy((cudaStream_t)s);
}

void mgcu_count_launch(long n) { g_launches += n; }

extern "C" long mgcu_launch_count(void) { return g_launches.load(); }
extern "C" double mgcu_device_free_bytes(void)
{
	size_t f = 0, t = 0;
	if (!mgcu_ctx() || cudaMemGetInfo(&f, &t) != cudaSuccess) return 0;
	return (double)f;
}

// ------------------------------------------------------------------------------------
// Peak arithmetic rates: every thread runs 8 independent FMA chains; the chains'
// results are stored so the compiler keeps the work.
// ------------------------------------------------------------------------------------
template <class F>
__global__ void __launch_bounds__(256) k_fma_peak(F* out, int iters, F a, F b)
{
	F x0 = (F)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
	for (int i = 0; i < iters; i++)
	{
#pragma unroll
		for (int u = 0; u < 16; u++)
		{
			x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
			x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
		}
	}
	out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <class F>
static double fma_peak(int iters)
{
	MgcuContext* c = mgcu_ctx();
	if (!c) return -1;
	const int blocks = c->nsm * 8, threads = 256;
	DevBuf out;
	if (out.alloc(sizeof(F) * blocks * threads)) return -1;
	float best = 1e30f;
	for (int rep = 0; rep < 4; rep++)
	{
		cudaEventRecord(c->ev0, c->stream);
		k_fma_peak<F><<<blocks, threads, 0, c->stream>>>(out.as<F>(), iters, (F)0.999999, (F)1e-7);
		mgcu_count_launch();
		cudaEventRecord(c->ev1, c->stream);
		if (cudaEventSynchronize(c->ev1) != cudaSuccess) return -1;
		float ms = 0;
		cudaEventElapsedTime(&ms, c->ev0, c->ev1);
		if (rep > 0 && ms < best) best = ms;
	}
	const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
	return flops / (best * 1e-3) / 1e9;
}

extern "C" double mgcu_fp32_peak_gflops(void) { return fma_peak<float>(4096); }
extern "C" double mgcu_fp64_peak_gflops(void) { return fma_peak<double>(64); }
