/*
 * U(2)+U(2) matchgate algebra in FP64, written once and compiled both as host C (the
 * ABI functions of matchgate.h) and as CUDA device code (projection, retraction and
 * the Hessian projection kernels).  Types are plain structs that share the memory
 * layout of C99 `double complex` and of the reference's struct matchgate
 * (src/matchgate.h:5-14: center block, then corner block, both row-major 2x2).
 */
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define MG_HD static __host__ __device__ __forceinline__
#else
#define MG_HD static inline
#endif

typedef struct { double re, im; } mgc;
typedef struct { mgc c[4]; mgc k[4]; } mgg;

MG_HD mgc mgc_make(double re, double im) { mgc z; z.re = re; z.im = im; return z; }
MG_HD mgc mgc_add(mgc a, mgc b) { return mgc_make(a.re + b.re, a.im + b.im); }
MG_HD mgc mgc_sub(mgc a, mgc b) { return mgc_make(a.re - b.re, a.im - b.im); }
MG_HD mgc mgc_mul(mgc a, mgc b) { return mgc_make(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
MG_HD mgc mgc_conj(mgc a) { return mgc_make(a.re, -a.im); }
MG_HD mgc mgc_scale(mgc a, double s) { return mgc_make(a.re * s, a.im * s); }
MG_HD double mgc_abs(mgc a) { return hypot(a.re, a.im); }

/* a / b by Smith's method (R. L. Smith, "Algorithm 116: Complex division",
 * Commun. ACM 5(8):435, 1962): scale by the larger component of b. */
MG_HD mgc mgc_div(mgc a, mgc b)
{
	if (fabs(b.re) >= fabs(b.im))
	{
		const double r = b.im / b.re, d = b.re + b.im * r;
		return mgc_make((a.re + a.im * r) / d, (a.im - a.re * r) / d);
	}
	else
	{
		const double r = b.re / b.im, d = b.re * r + b.im;
		return mgc_make((a.re * r + a.im) / d, (a.im * r - a.re) / d);
	}
}

/* ---- 2x2 blocks ---- */

/* c = a b, accumulating as in src/matchgate.c:338-352 */
MG_HD void mg2_mul(const mgc* a, const mgc* b, mgc* c)
{
	mgc r[4];
	for (int i = 0; i < 2; i++)
		for (int k = 0; k < 2; k++)
			r[2 * i + k] = mgc_add(mgc_mul(a[2 * i], b[k]), mgc_mul(a[2 * i + 1], b[2 + k]));
	for (int q = 0; q < 4; q++) c[q] = r[q];
}

/* 2x2 inverse by Gauss-Jordan elimination with partial pivoting (the method of
 * src/matchgate.c:414-479); returns -1 for a singular block */
MG_HD int mg2_inv(const mgc* a, mgc* out)
{
	mgc m[4] = { a[0], a[1], a[2], a[3] };
	mgc v[4] = { mgc_make(1, 0), mgc_make(0, 0), mgc_make(0, 0), mgc_make(1, 0) };
	for (int k = 0; k < 2; k++)
	{
		int piv = k;
		double p = mgc_abs(m[2 * k + k]);
		if (k == 0 && mgc_abs(m[2]) > p) { piv = 1; p = mgc_abs(m[2]); }
		if (p == 0) return -1;
		if (piv != k)
			for (int c = 0; c < 2; c++)
			{
				mgc s = m[2 * k + c]; m[2 * k + c] = m[2 * piv + c]; m[2 * piv + c] = s;
				s = v[2 * k + c]; v[2 * k + c] = v[2 * piv + c]; v[2 * piv + c] = s;
			}
		const int o = 1 - k;
		const mgc f = mgc_div(m[2 * o + k], m[2 * k + k]);
		for (int c = k + 1; c < 2; c++) m[2 * o + c] = mgc_sub(m[2 * o + c], mgc_mul(f, m[2 * k + c]));
		m[2 * o + k] = mgc_make(0, 0);
		for (int c = 0; c < 2; c++) v[2 * o + c] = mgc_sub(v[2 * o + c], mgc_mul(f, v[2 * k + c]));
		for (int c = k + 1; c < 2; c++) m[2 * k + c] = mgc_div(m[2 * k + c], m[2 * k + k]);
		for (int c = 0; c < 2; c++) v[2 * k + c] = mgc_div(v[2 * k + c], m[2 * k + k]);
		m[2 * k + k] = mgc_make(1, 0);
	}
	for (int q = 0; q < 4; q++) out[q] = v[q];
	return 0;
}

/* ---- matchgates ---- */

MG_HD void mgg_zero(mgg* a) { for (int q = 0; q < 4; q++) { a->c[q] = mgc_make(0, 0); a->k[q] = mgc_make(0, 0); } }
MG_HD void mgg_identity(mgg* a)
{
	mgg_zero(a);
	a->c[0] = a->c[3] = a->k[0] = a->k[3] = mgc_make(1, 0);
}
MG_HD void mgg_mul(const mgg* a, const mgg* b, mgg* c)
{
	mgg r;
	mg2_mul(a->c, b->c, r.c);
	mg2_mul(a->k, b->k, r.k);
	*c = r;
}
MG_HD void mgg_add(mgg* a, const mgg* b) { for (int q = 0; q < 4; q++) { a->c[q] = mgc_add(a->c[q], b->c[q]); a->k[q] = mgc_add(a->k[q], b->k[q]); } }
MG_HD void mgg_sub(mgg* a, const mgg* b) { for (int q = 0; q < 4; q++) { a->c[q] = mgc_sub(a->c[q], b->c[q]); a->k[q] = mgc_sub(a->k[q], b->k[q]); } }
MG_HD void mgg_scale(mgg* a, double s) { for (int q = 0; q < 4; q++) { a->c[q] = mgc_scale(a->c[q], s); a->k[q] = mgc_scale(a->k[q], s); } }
MG_HD void mgg_conj(mgg* a) { for (int q = 0; q < 4; q++) { a->c[q] = mgc_conj(a->c[q]); a->k[q] = mgc_conj(a->k[q]); } }
MG_HD void mgg_transpose(const mgg* a, mgg* at)
{
	mgg r;
	for (int i = 0; i < 2; i++)
		for (int j = 0; j < 2; j++) { r.c[2 * i + j] = a->c[2 * j + i]; r.k[2 * i + j] = a->k[2 * j + i]; }
	*at = r;
}
MG_HD void mgg_adjoint(const mgg* a, mgg* ah)
{
	mgg r;
	for (int i = 0; i < 2; i++)
		for (int j = 0; j < 2; j++) { r.c[2 * i + j] = mgc_conj(a->c[2 * j + i]); r.k[2 * i + j] = mgc_conj(a->k[2 * j + i]); }
	*ah = r;
}

/* Hermitian part of each block (src/matchgate.c:196-212) */
MG_HD void mgg_symm(const mgg* w, mgg* z)
{
	mgg r;
	r.k[0] = mgc_make(w->k[0].re, 0); r.c[0] = mgc_make(w->c[0].re, 0);
	r.c[3] = mgc_make(w->c[3].re, 0); r.k[3] = mgc_make(w->k[3].re, 0);
	r.k[1] = mgc_scale(mgc_add(w->k[1], mgc_conj(w->k[2])), 0.5);
	r.c[1] = mgc_scale(mgc_add(w->c[1], mgc_conj(w->c[2])), 0.5);
	r.k[2] = mgc_conj(r.k[1]);
	r.c[2] = mgc_conj(r.c[1]);
	*z = r;
}

/* anti-Hermitian part of each block (src/matchgate.c:219-243) */
MG_HD void mgg_antisymm(const mgg* w, mgg* z)
{
	mgg r;
	r.k[0] = mgc_make(0, w->k[0].im); r.c[0] = mgc_make(0, w->c[0].im);
	r.c[3] = mgc_make(0, w->c[3].im); r.k[3] = mgc_make(0, w->k[3].im);
	r.k[1] = mgc_scale(mgc_sub(w->k[1], mgc_conj(w->k[2])), 0.5);
	r.c[1] = mgc_scale(mgc_sub(w->c[1], mgc_conj(w->c[2])), 0.5);
	r.k[2] = mgc_scale(mgc_conj(r.k[1]), -1.0);
	r.c[2] = mgc_scale(mgc_conj(r.c[1]), -1.0);
	*z = r;
}

/* 8 reals -> anti-Hermitian U(2)+U(2) element (src/matchgate.c:251-270) */
MG_HD void mgg_real_to_antisymm(const double* r, mgg* w)
{
	w->c[0] = mgc_make(0, r[0]);
	w->c[3] = mgc_make(0, r[3]);
	w->k[0] = mgc_make(0, r[4]);
	w->k[3] = mgc_make(0, r[7]);
	w->c[1] = mgc_make(0.5 * (r[1] - r[2]), 0.5 * (r[1] + r[2]));
	w->k[1] = mgc_make(0.5 * (r[5] - r[6]), 0.5 * (r[5] + r[6]));
	w->c[2] = mgc_scale(mgc_conj(w->c[1]), -1.0);
	w->k[2] = mgc_scale(mgc_conj(w->k[1]), -1.0);
}

/* inverse isometry (src/matchgate.c:277-288) */
MG_HD void mgg_antisymm_to_real(const mgg* w, double* r)
{
	for (int q = 0; q < 4; q++)
	{
		r[q]     = w->c[q].re + w->c[q].im;
		r[q + 4] = w->k[q].re + w->k[q].im;
	}
}

/* z = v A(r) (src/matchgate.c:296-301) */
MG_HD void mgg_real_to_tangent(const double* r, const mgg* v, mgg* z)
{
	mgg a;
	mgg_real_to_antisymm(r, &a);
	mgg_mul(v, &a, z);
}

/* r = real(antisymm(v^H z)) (src/matchgate.c:309-316) */
MG_HD void mgg_tangent_to_real(const mgg* v, const mgg* z, double* r)
{
	mgg w, t;
	mgg_adjoint(v, &w);
	mgg_mul(&w, z, &t);
	mgg_antisymm(&t, &w);
	mgg_antisymm_to_real(&w, r);
}

/* p = z - u symm(u^H z) (src/matchgate.c:323-334) */
MG_HD void mgg_project_tangent(const mgg* u, const mgg* z, mgg* p)
{
	mgg v, w;
	mgg_adjoint(u, &v);
	mgg_mul(&v, z, &w);
	mgg_symm(&w, &v);
	mgg_mul(u, &v, &w);
	mgg r = *z;
	mgg_sub(&r, &w);
	*p = r;
}

/* (a b c + c b a) / 2 (src/matchgate.c:381-393) */
MG_HD void mgg_sym_triple(const mgg* a, const mgg* b, const mgg* c, mgg* ret)
{
	mgg u, v, r;
	mgg_mul(a, b, &u);
	mgg_mul(&u, c, &r);
	mgg_mul(c, b, &u);
	mgg_mul(&u, a, &v);
	mgg_add(&r, &v);
	mgg_scale(&r, 0.5);
	*ret = r;
}

MG_HD int mgg_inverse(const mgg* a, mgg* ainv)
{
	mgg r;
	const int e1 = mg2_inv(a->c, r.c);
	const int e2 = mg2_inv(a->k, r.k);
	*ainv = r;
	return (e1 || e2) ? -1 : 0;
}

MG_HD double mg_unif_dist4(const mgc* a, const mgc* b)
{
	double d = 0;
	for (int q = 0; q < 4; q++) d = fmax(d, mgc_abs(mgc_sub(a[q], b[q])));
	return d;
}

/* unitary polar factor by the Newton iteration u <- (u + u^{-H})/2 per block
 * (Higham 1986), at most 14 steps, stopping from step 4 on once a step changes
 * the blocks by less than 1e-14 (src/matchgate.c:517-541) */
MG_HD void mgg_polar(const mgg* a, mgg* u)
{
	mgg cur = *a;
	for (int it = 0; it < 14; it++)
	{
		mgg inv, w;
		mgg_inverse(&cur, &inv);
		mgg_adjoint(&inv, &w);
		mgg_add(&cur, &w);
		mgg_scale(&cur, 0.5);
		if (it >= 4 && mg_unif_dist4(cur.c, w.c) < 1e-14 && mg_unif_dist4(cur.k, w.k) < 1e-14) break;
	}
	*u = cur;
}

/* v = polar(u (I + A(eta))) (src/matchgate.c:548-562) */
MG_HD void mgg_retract(const mgg* u, const double* eta, mgg* v)
{
	mgg z, w;
	mgg_real_to_antisymm(eta, &z);
	z.k[0].re += 1; z.c[0].re += 1; z.c[3].re += 1; z.k[3].re += 1;
	mgg_mul(u, &z, &w);
	mgg_polar(&w, v);
}

/* One 8-column block of the real Riemannian Hessian (src/matchgate_target.c:910-961):
 * for layer pair (i, j) and unit tangent direction k at gate j, given the complex
 * Hessian blocks hij (8x8 row-major, rows x of layer i, columns y of layer j),
 * returns the 8 reals of column k.  dvc_i is the conjugated gradient of gate i. */
MG_HD void mg_project_hessian_column(const mgg* vi, const mgg* vj, const mgg* dvc_i, int same_layer,
	const mgc* hij, int k, double* out8)
{
	double r[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
	r[k] = 1;
	mgg Z, G;
	mgg_real_to_tangent(r, vj, &Z);
	mgg_zero(&G);
	for (int x = 0; x < 4; x++)
		for (int y = 0; y < 4; y++)
		{
			G.c[x] = mgc_add(G.c[x], mgc_add(mgc_mul(hij[x * 8 + y], Z.c[y]), mgc_mul(hij[x * 8 + y + 4], Z.k[y])));
			G.k[x] = mgc_add(G.k[x], mgc_add(mgc_mul(hij[(x + 4) * 8 + y], Z.c[y]), mgc_mul(hij[(x + 4) * 8 + y + 4], Z.k[y])));
		}
	mgg_conj(&G);
	if (same_layer)
	{
		mgg P, gh, T;
		mgg_project_tangent(vi, &G, &P);
		mgg_adjoint(dvc_i, &gh);
		mgg_sym_triple(&Z, &gh, vi, &T);
		mgg_sub(&P, &T);
		G = P;
	}
	mgg_tangent_to_real(vi, &G, out8);
}
