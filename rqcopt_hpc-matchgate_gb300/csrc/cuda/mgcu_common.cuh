// Shared CUDA definitions: runtime context, error handling, and the three precision
// policies of the sweep engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../mg_internal.h"

// ------------------------------------------------------------------------------------
// runtime context (mgcu_runtime.cu)
// ------------------------------------------------------------------------------------
struct MgcuContext
{
	int device;
	int nsm;
	size_t smem_optin;
	cudaStream_t stream;
	cudaEvent_t ev0, ev1;
};

MgcuContext* mgcu_ctx();                 // initialises on first use; NULL on failure
cudaStream_t mgcu_stream();              // the calling host thread's stream (default: the library's)
void mgcu_count_launch(long n = 1);
int mgcu_check(cudaError_t e, const char* what, const char* file, int line);

#define MGCU_TRY(call) do { cudaError_t _e = (call); if (_e != cudaSuccess) return mgcu_check(_e, #call, __FILE__, __LINE__); } while (0)
#define MGCU_LAUNCHED() do { mgcu_count_launch(); cudaError_t _e = cudaGetLastError(); if (_e != cudaSuccess) return mgcu_check(_e, "kernel launch", __FILE__, __LINE__); } while (0)

// simple RAII device buffer
struct DevBuf
{
	void* p = nullptr;
	size_t n = 0;
	DevBuf() = default;
	DevBuf(const DevBuf&) = delete;
	DevBuf& operator=(const DevBuf&) = delete;
	~DevBuf() { if (p) cudaFree(p); }
	int alloc(size_t bytes)
	{
		if (bytes <= n && p) return 0;
		if (p) { cudaFree(p); p = nullptr; n = 0; }
		if (bytes == 0) bytes = 16;
		cudaError_t e = cudaMalloc(&p, bytes);
		if (e != cudaSuccess) { p = nullptr; mgcu_check(e, "cudaMalloc", __FILE__, __LINE__); return MG_ERR_ALLOC; }
		n = bytes;
		return 0;
	}
	void release()
	{
		if (p) cudaFree(p);
		p = nullptr;
		n = 0;
	}
	template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

// ------------------------------------------------------------------------------------
// float-float arithmetic (pairs of FP32 with |lo| <= ulp(hi)/2).  Error-free
// transformations after Knuth (TwoSum), Dekker (FastTwoSum) and the FMA-based
// TwoProduct; compensated dot products after Ogita, Rump and Oishi, "Accurate sum
// and dot product", SIAM J. Sci. Comput. 26(6), 2005.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
	s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e)
{
	s = __fadd_rn(a, b);
	e = __fsub_rn(b, __fsub_rn(s, a));
}

// (ah + al)(bh + bl) = p + e up to O(u^2), lo*lo dropped
__device__ __forceinline__ void ff_prod(float ah, float al, float bh, float bl, float& p, float& e)
{
	p = __fmul_rn(ah, bh);
	e = __fmaf_rn(ah, bh, -p);
	e = __fmaf_rn(ah, bl, e);
	e = __fmaf_rn(al, bh, e);
}

// running compensated sum (sh, sl) += (ah+al)(bh+bl)
__device__ __forceinline__ void ff_acc_prod(float& sh, float& sl, float ah, float al, float bh, float bl)
{
	float p, e, s, t;
	ff_prod(ah, al, bh, bl, p, e);
	two_sum(sh, p, s, t);
	sh = s;
	sl = __fadd_rn(sl, __fadd_rn(t, e));
}

// (ah, al) += (bh, bl), renormalised
__device__ __forceinline__ void ff_add(float& ah, float& al, float bh, float bl)
{
	float s, t;
	two_sum(ah, bh, s, t);
	t = __fadd_rn(t, __fadd_rn(al, bl));
	fast_two_sum(s, t, ah, al);
}

// ------------------------------------------------------------------------------------
// Precision policies.  Each defines
//   T      state / gate element (one complex number)
//   Acc    complex accumulator used for overlaps and gradient sums
//   madd2  a x + b y (complex)
//   acc_*  compensated accumulation of complex products
//   to_d   accumulator -> FP64 parts
// ------------------------------------------------------------------------------------

// plain complex128
struct PrecD
{
	typedef double2 T;
	struct Acc { double re, im; };
	static constexpr int kId = MG_PREC_FP64_ID;
	__host__ __device__ static T make(double re, double im) { return make_double2(re, im); }
	__device__ static T zero() { return make_double2(0.0, 0.0); }
	__device__ static T madd2(T a, T x, T b, T y)
	{
		T r;
		r.x = fma(a.x, x.x, fma(-a.y, x.y, fma(b.x, y.x, -b.y * y.y)));
		r.y = fma(a.x, x.y, fma(a.y, x.x, fma(b.x, y.y, b.y * y.x)));
		return r;
	}
	__device__ static T negconj(T a) { return make_double2(-a.x, a.y); }
	__device__ static T neg(T a) { return make_double2(-a.x, -a.y); }
	__device__ static T add(T a, T b) { return make_double2(a.x + b.x, a.y + b.y); }
	// a with its sign flipped when s == 1 (bit operations, no arithmetic)
	__device__ static T negif(T a, unsigned s)
	{
		const long long m = (long long)s << 63;
		return make_double2(__longlong_as_double(__double_as_longlong(a.x) ^ m), __longlong_as_double(__double_as_longlong(a.y) ^ m));
	}
	__device__ static T mul(T a, T x) { return make_double2(fma(a.x, x.x, -a.y * x.y), fma(a.x, x.y, a.y * x.x)); }
	// a x + b y for entries that are real or imaginary: a = (c_re, c_im) with c_re, c_im the
	// coefficients of the (possibly swapped) components of x; swap when the entry is imaginary
	__device__ static T madd2_ri(T a, bool ra, T x, T b, bool rb, T y)
	{
		const double xr = ra ? x.y : x.x, xi = ra ? x.x : x.y, yr = rb ? y.y : y.x, yi = rb ? y.x : y.y;
		return make_double2(fma(a.x, xr, b.x * yr), fma(a.y, xi, b.y * yi));
	}
	// symmetric hop block [[c, i s], [i s, c]] (c, s real) on the pair (a, b), its
	// off-diagonal entries negated when sg == 1; c0 and c1 are the staged block entries
	// (real c stored as (c, c), imaginary i s as (-s, s))
	__device__ static void hop(T c0, T c1, unsigned sg, T& a, T& b)
	{
		const double c = c0.x, s = __longlong_as_double(__double_as_longlong(c1.y) ^ ((long long)sg << 63));
		const T x = a, y = b;
		a = make_double2(fma(c, x.x, -s * y.y), fma(c, x.y, s * y.x));
		b = make_double2(fma(c, y.x, -s * x.y), fma(c, y.y, s * x.x));
	}
	__device__ static Acc acc_zero() { Acc a; a.re = 0; a.im = 0; return a; }
	__device__ static void acc_mul_add(Acc& s, T d, T x)
	{
		s.re = fma(d.x, x.x, fma(-d.y, x.y, s.re));
		s.im = fma(d.x, x.y, fma(d.y, x.x, s.im));
	}
	// short sums (a few quartets per thread, then a block reduction): same as acc_mul_add
	__device__ static void acc_mul_add_short(Acc& s, T d, T x) { acc_mul_add(s, d, x); }
	__device__ static void acc_add(Acc& s, const Acc& o) { s.re += o.re; s.im += o.im; }
	__device__ static Acc shfl_xor(const Acc& a, int m)
	{
		Acc r;
		r.re = __shfl_xor_sync(0xffffffffu, a.re, m);
		r.im = __shfl_xor_sync(0xffffffffu, a.im, m);
		return r;
	}
	__device__ static double2 to_d(const Acc& a) { return make_double2(a.re, a.im); }
};

// complex FP32 sweeps, compensated FP32 sums
struct PrecF
{
	typedef float2 T;
	struct Acc { float rh, rl, ih, il; };
	static constexpr int kId = MG_PREC_FP32_ID;
	__host__ __device__ static T make(double re, double im) { return make_float2((float)re, (float)im); }
	__device__ static T zero() { return make_float2(0.f, 0.f); }
	__device__ static T madd2(T a, T x, T b, T y)
	{
		T r;
		r.x = fmaf(a.x, x.x, fmaf(-a.y, x.y, fmaf(b.x, y.x, -b.y * y.y)));
		r.y = fmaf(a.x, x.y, fmaf(a.y, x.x, fmaf(b.x, y.y, b.y * y.x)));
		return r;
	}
	__device__ static T negconj(T a) { return make_float2(-a.x, a.y); }
	__device__ static T neg(T a) { return make_float2(-a.x, -a.y); }
	__device__ static T add(T a, T b) { return make_float2(a.x + b.x, a.y + b.y); }
	__device__ static T negif(T a, unsigned s)
	{
		const unsigned m = s << 31;
		return make_float2(__uint_as_float(__float_as_uint(a.x) ^ m), __uint_as_float(__float_as_uint(a.y) ^ m));
	}
	__device__ static T mul(T a, T x) { return make_float2(fmaf(a.x, x.x, -a.y * x.y), fmaf(a.x, x.y, a.y * x.x)); }
	__device__ static T madd2_ri(T a, bool ra, T x, T b, bool rb, T y)
	{
		const float xr = ra ? x.y : x.x, xi = ra ? x.x : x.y, yr = rb ? y.y : y.x, yi = rb ? y.x : y.y;
		return make_float2(fmaf(a.x, xr, b.x * yr), fmaf(a.y, xi, b.y * yi));
	}
	__device__ static void hop(T c0, T c1, unsigned sg, T& a, T& b)
	{
		const float c = c0.x, s = __uint_as_float(__float_as_uint(c1.y) ^ (sg << 31));
		const T x = a, y = b;
		a = make_float2(fmaf(c, x.x, -s * y.y), fmaf(c, x.y, s * y.x));
		b = make_float2(fmaf(c, y.x, -s * x.y), fmaf(c, y.y, s * x.x));
	}
	__device__ static Acc acc_zero() { Acc a; a.rh = a.rl = a.ih = a.il = 0.f; return a; }
	__device__ static void acc_mul_add(Acc& s, T d, T x)
	{
		// products rounded once in FP32, then summed without further rounding loss
		const float pr = fmaf(d.x, x.x, -d.y * x.y);
		const float pi = fmaf(d.x, x.y, d.y * x.x);
		float t, e;
		two_sum(s.rh, pr, t, e); s.rh = t; s.rl += e;
		two_sum(s.ih, pi, t, e); s.ih = t; s.il += e;
	}
	__device__ static void acc_mul_add_short(Acc& s, T d, T x) { acc_mul_add(s, d, x); }
	__device__ static void acc_add(Acc& s, const Acc& o) { ff_add(s.rh, s.rl, o.rh, o.rl); ff_add(s.ih, s.il, o.ih, o.il); }
	__device__ static Acc shfl_xor(const Acc& a, int m)
	{
		Acc r;
		r.rh = __shfl_xor_sync(0xffffffffu, a.rh, m); r.rl = __shfl_xor_sync(0xffffffffu, a.rl, m);
		r.ih = __shfl_xor_sync(0xffffffffu, a.ih, m); r.il = __shfl_xor_sync(0xffffffffu, a.il, m);
		return r;
	}
	__device__ static double2 to_d(const Acc& a) { return make_double2((double)a.rh + (double)a.rl, (double)a.ih + (double)a.il); }
};

// float-float complex sweeps ("mixed"): T = (re_hi, im_hi, re_lo, im_lo)
// Float-float complex numbers (re_hi, im_hi, re_lo, im_lo).  Results of madd2 / mul /
// madd2_ri are not renormalised: hi is the rounded sum of the hi products and lo collects
// the exact product and sum errors and the lo cross terms, so |lo| stays within a few
// units in the last place of the inputs' magnitude and hi + lo carries about 44
// significant bits; every consumer uses hi + lo, never hi alone.
struct PrecX
{
	typedef float4 T;
	typedef PrecF::Acc Acc;
	static constexpr int kId = MG_PREC_MIXED_ID;
	__host__ __device__ static T make(double re, double im)
	{
		const float rh = (float)re, ih = (float)im;
		return make_float4(rh, ih, (float)(re - (double)rh), (float)(im - (double)ih));
	}
	__device__ static T zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
	// a x + b y with every real part summed as a 4-term compensated dot product
	__device__ static T madd2(T a, T x, T b, T y)
	{
		float rh, rl, ih, il;
		// real: a.re x.re - a.im x.im + b.re y.re - b.im y.im
		ff_prod(a.x, a.z, x.x, x.z, rh, rl);
		ff_acc_prod(rh, rl, -a.y, -a.w, x.y, x.w);
		ff_acc_prod(rh, rl, b.x, b.z, y.x, y.z);
		ff_acc_prod(rh, rl, -b.y, -b.w, y.y, y.w);
		// imag: a.re x.im + a.im x.re + b.re y.im + b.im y.re
		ff_prod(a.x, a.z, x.y, x.w, ih, il);
		ff_acc_prod(ih, il, a.y, a.w, x.x, x.z);
		ff_acc_prod(ih, il, b.x, b.z, y.y, y.w);
		ff_acc_prod(ih, il, b.y, b.w, y.x, y.z);
		return make_float4(rh, ih, rl, il);
	}
	__device__ static T negconj(T a) { return make_float4(-a.x, a.y, -a.z, a.w); }
	__device__ static T neg(T a) { return make_float4(-a.x, -a.y, -a.z, -a.w); }
	// a + b: hi = the rounded sum of the hi parts, lo = its exact error plus both lo parts
	__device__ static T add(T a, T b)
	{
		float rh, re, ih, ie;
		two_sum(a.x, b.x, rh, re);
		two_sum(a.y, b.y, ih, ie);
		return make_float4(rh, ih, __fadd_rn(re, __fadd_rn(a.z, b.z)), __fadd_rn(ie, __fadd_rn(a.w, b.w)));
	}
	__device__ static T negif(T a, unsigned s)
	{
		const unsigned m = s << 31;
		return make_float4(__uint_as_float(__float_as_uint(a.x) ^ m), __uint_as_float(__float_as_uint(a.y) ^ m),
			__uint_as_float(__float_as_uint(a.z) ^ m), __uint_as_float(__float_as_uint(a.w) ^ m));
	}
	// a x as two 2-term compensated dot products
	__device__ static T mul(T a, T x)
	{
		float rh, rl, ih, il;
		ff_prod(a.x, a.z, x.x, x.z, rh, rl);
		ff_acc_prod(rh, rl, -a.y, -a.w, x.y, x.w);
		ff_prod(a.x, a.z, x.y, x.w, ih, il);
		ff_acc_prod(ih, il, a.y, a.w, x.x, x.z);
		return make_float4(rh, ih, rl, il);
	}
	// a x + b y for real-or-imaginary entries (see PrecD::madd2_ri): 2-term dots per part
	__device__ static T madd2_ri(T a, bool ra, T x, T b, bool rb, T y)
	{
		const float xrh = ra ? x.y : x.x, xrl = ra ? x.w : x.z, xih = ra ? x.x : x.y, xil = ra ? x.z : x.w;
		const float yrh = rb ? y.y : y.x, yrl = rb ? y.w : y.z, yih = rb ? y.x : y.y, yil = rb ? y.z : y.w;
		float rh, rl, ih, il;
		ff_prod(a.x, a.z, xrh, xrl, rh, rl);
		ff_acc_prod(rh, rl, b.x, b.z, yrh, yrl);
		ff_prod(a.y, a.w, xih, xil, ih, il);
		ff_acc_prod(ih, il, b.y, b.w, yih, yil);
		return make_float4(rh, ih, rl, il);
	}
	// symmetric hop block: every output a 2-term compensated dot with coefficients (c, +-s);
	// the string sign flips s (two sign bits), not the inputs
	__device__ static void hop(T c0, T c1, unsigned sg, T& a, T& b)
	{
		const float ch = c0.x, cl = c0.z;
		const float sh = __uint_as_float(__float_as_uint(c1.y) ^ (sg << 31)), sl = __uint_as_float(__float_as_uint(c1.w) ^ (sg << 31));
		const T x = a, y = b;
		float rh, rl, ih, il;
		ff_prod(ch, cl, x.x, x.z, rh, rl);
		ff_acc_prod(rh, rl, -sh, -sl, y.y, y.w);
		ff_prod(ch, cl, x.y, x.w, ih, il);
		ff_acc_prod(ih, il, sh, sl, y.x, y.z);
		a = make_float4(rh, ih, rl, il);
		ff_prod(ch, cl, y.x, y.z, rh, rl);
		ff_acc_prod(rh, rl, -sh, -sl, x.y, x.w);
		ff_prod(ch, cl, y.y, y.w, ih, il);
		ff_acc_prod(ih, il, sh, sl, x.x, x.z);
		b = make_float4(rh, ih, rl, il);
	}
	__device__ static Acc acc_zero() { return PrecF::acc_zero(); }
	__device__ static void acc_mul_add(Acc& s, T d, T x)
	{
		ff_acc_prod(s.rh, s.rl, d.x, d.z, x.x, x.z);
		ff_acc_prod(s.rh, s.rl, -d.y, -d.w, x.y, x.w);
		ff_acc_prod(s.ih, s.il, d.x, d.z, x.y, x.w);
		ff_acc_prod(s.ih, s.il, d.y, d.w, x.x, x.z);
		float a, b;
		fast_two_sum(s.rh, s.rl, a, b); s.rh = a; s.rl = b;
		fast_two_sum(s.ih, s.il, a, b); s.ih = a; s.il = b;
	}
	// the same without renormalising, for sums of at most a few hundred products that are
	// renormalised when reduced (ff_add): hi is the rounded sum of the exact hi products,
	// lo collects every rounding error, and |lo| <= n ulp(hi) keeps hi + lo within
	// n 2^-48 of the exact sum relative to hi
	__device__ static void acc_mul_add_short(Acc& s, T d, T x)
	{
		ff_acc_prod(s.rh, s.rl, d.x, d.z, x.x, x.z);
		ff_acc_prod(s.rh, s.rl, -d.y, -d.w, x.y, x.w);
		ff_acc_prod(s.ih, s.il, d.x, d.z, x.y, x.w);
		ff_acc_prod(s.ih, s.il, d.y, d.w, x.x, x.z);
	}
	__device__ static void acc_add(Acc& s, const Acc& o) { PrecF::acc_add(s, o); }
	__device__ static Acc shfl_xor(const Acc& a, int m) { return PrecF::shfl_xor(a, m); }
	__device__ static double2 to_d(const Acc& a) { return PrecF::to_d(a); }
};
