/*
 * Target construction: Suzuki product-formula circuits of the spinful 1-D Fermi-Hubbard
 * model from matchgates (the reference builds these targets in Python,
 * benchmark_hpc/spl_hubbard1d_bench_init.py:24-118 with the product rules of
 * test/rqcopt_matfree/splitting_method.py:161-193).
 *
 * Model: open chain of nsites sites, qubits interleaved (2s = site s spin up, 2s+1 = spin
 * down), Jordan-Wigner encoded; H = A + B + C with A = U sum_s n_up n_down (on-site), B and C
 * the hops -J (c^dag c + h.c.) of both spins on the even and odd bonds.  A same-spin hop
 * between sites s, s+1 (qubits 2s, 2s+2 or 2s+1, 2s+3) is a nearest-neighbour matchgate after
 * a fermionic swap of the two middle qubits (2s+1, 2s+2), which is undone afterwards.
 *
 * Product rule: Suzuki's symmetric formula of order 2k on the terms (A, B, C):
 * S_2(h) = A(h/2) B(h/2) C(h) B(h/2) A(h/2) and S_2k(h) = S_2k-2(p h)^2 S_2k-2((1-4p) h)
 * S_2k-2(p h)^2 with p = 1 / (4 - 4^(1/(2k-1))) (M. Suzuki, Phys. Lett. A 146, 319 (1990));
 * neighbouring layers of the same term are merged, also across the nsteps steps of size
 * h = t / nsteps, and then neighbouring gates on the same wire pair are multiplied.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mg_gb300.h"
#include "../mg_internal.h"

typedef struct { int* term; double* coeff; int n, cap; } rule_t;

static int rule_push(rule_t* r, int term, double c)
{
	if (r->n > 0 && r->term[r->n - 1] == term) { r->coeff[r->n - 1] += c; return 0; }
	if (r->n == r->cap)
	{
		const int nc = r->cap ? 2 * r->cap : 16;
		int* t = realloc(r->term, sizeof(int) * nc);
		if (!t) return -1;
		r->term = t;
		double* c2 = realloc(r->coeff, sizeof(double) * nc);
		if (!c2) return -1;
		r->coeff = c2;
		r->cap = nc;
	}
	r->term[r->n] = term; r->coeff[r->n] = c; r->n++;
	return 0;
}

/* the layers of S_2k(scale) over nterms terms appended to r: S_2 = the terms forward then
 * backward, each with coefficient 1/2 (the middle term's two halves merge) */
static int suzuki(rule_t* r, int k, double scale, int nterms)
{
	if (k == 1)
	{
		for (int i = 0; i < nterms; i++) if (rule_push(r, i, 0.5 * scale)) return -1;
		for (int i = nterms - 1; i >= 0; i--) if (rule_push(r, i, 0.5 * scale)) return -1;
		return 0;
	}
	const double p = 1.0 / (4.0 - pow(4.0, 1.0 / (2 * k - 1)));
	const double w[5] = { p, p, 1 - 4 * p, p, p };
	for (int i = 0; i < 5; i++) if (suzuki(r, k - 1, w[i] * scale, nterms)) return -1;
	return 0;
}

typedef struct { struct matchgate* g; int* w; int n, cap; } gates_t;

static struct matchgate mk(numeric c0, numeric c1, numeric c2, numeric c3, numeric k0, numeric k1, numeric k2, numeric k3)
{
	struct matchgate m;
	m.center_block.data[0] = c0; m.center_block.data[1] = c1; m.center_block.data[2] = c2; m.center_block.data[3] = c3;
	m.corner_block.data[0] = k0; m.corner_block.data[1] = k1; m.corner_block.data[2] = k2; m.corner_block.data[3] = k3;
	return m;
}

static void mul2(const numeric* b, const numeric* a, numeric* out)
{
	numeric r[4];
	r[0] = b[0] * a[0] + b[1] * a[2]; r[1] = b[0] * a[1] + b[1] * a[3];
	r[2] = b[2] * a[0] + b[3] * a[2]; r[3] = b[2] * a[1] + b[3] * a[3];
	memcpy(out, r, sizeof(r));
}

/* append a gate on wires (i, j); a gate following one on the same ordered pair is
 * multiplied into it (later times earlier, both blocks) */
static int push_gate(gates_t* s, struct matchgate g, int i, int j)
{
	if (s->n > 0 && s->w[2 * (s->n - 1)] == i && s->w[2 * (s->n - 1) + 1] == j)
	{
		struct matchgate* a = &s->g[s->n - 1];
		mul2(g.center_block.data, a->center_block.data, a->center_block.data);
		mul2(g.corner_block.data, a->corner_block.data, a->corner_block.data);
		return 0;
	}
	if (s->n == s->cap)
	{
		const int nc = s->cap ? 2 * s->cap : 256;
		struct matchgate* g2 = realloc(s->g, sizeof(struct matchgate) * nc);
		if (!g2) return -1;
		s->g = g2;
		int* w2 = realloc(s->w, sizeof(int) * 2 * nc);
		if (!w2) return -1;
		s->w = w2;
		s->cap = nc;
	}
	s->g[s->n] = g; s->w[2 * s->n] = i; s->w[2 * s->n + 1] = j; s->n++;
	return 0;
}

static int hubbard_build(int nsites, double J, double U, double t, int nsteps, int order, gates_t* out)
{
	if (nsites < 2 || nsites > 16 || nsteps < 1 || order < 2 || order % 2 || order > 12)
	{
		mg_set_error("Hubbard circuit: need 2 <= nsites <= 16, nsteps >= 1 and an even order 2..12");
		return MG_ERR_ARG;
	}
	rule_t r = { 0 };
	const double h = t / nsteps;
	for (int s = 0; s < nsteps; s++)
		if (suzuki(&r, order / 2, h, 3)) { free(r.term); free(r.coeff); return -1; }
	const struct matchgate fswap = mk(0, 1, 1, 0, 1, 0, 0, -1);
	int rc = 0;
	for (int l = 0; l < r.n && !rc; l++)
	{
		const double tau = r.coeff[l];
		if (r.term[l] == 0)
		{
			const struct matchgate g = mk(1, 0, 0, 1, 1, 0, 0, cexp(-I * U * tau));
			for (int s = 0; s < nsites && !rc; s++) rc = push_gate(out, g, 2 * s, 2 * s + 1);
			continue;
		}
		const int parity = r.term[l] - 1;
		const double c = cos(J * tau), sn = sin(J * tau);
		const struct matchgate hop = mk(c, I * sn, I * sn, c, 1, 0, 0, 1);
		for (int s = parity; s < nsites - 1 && !rc; s += 2) rc = push_gate(out, fswap, 2 * s + 1, 2 * s + 2);
		for (int s = parity; s < nsites - 1 && !rc; s += 2)
		{
			rc = push_gate(out, hop, 2 * s, 2 * s + 1);
			if (!rc) rc = push_gate(out, hop, 2 * s + 2, 2 * s + 3);
		}
		for (int s = parity; s < nsites - 1 && !rc; s += 2) rc = push_gate(out, fswap, 2 * s + 1, 2 * s + 2);
	}
	free(r.term); free(r.coeff);
	return rc;
}

int mg_hubbard_trotter_circuit(int nsites, double J, double U, double t, int nsteps, int order,
	struct matchgate gates[], int wires[], int capacity)
{
	gates_t s = { 0 };
	const int rc = hubbard_build(nsites, J, U, t, nsteps, order, &s);
	if (rc) { free(s.g); free(s.w); return rc; }
	if (gates && wires && capacity >= s.n)
	{
		memcpy(gates, s.g, sizeof(struct matchgate) * s.n);
		memcpy(wires, s.w, sizeof(int) * 2 * s.n);
	}
	const int n = s.n;
	free(s.g); free(s.w);
	return n;
}

void* mg_target_hubbard(int nsites, double J, double U, double t, int nsteps, int order)
{
	gates_t s = { 0 };
	if (hubbard_build(nsites, J, U, t, nsteps, order, &s)) { free(s.g); free(s.w); return NULL; }
	void* h = mg_target_circuit(s.g, s.n, s.w, 2 * nsites);
	free(s.g); free(s.w);
	return h;
}

/*
 * The spinless 1-D Fermi-Hubbard brickwall of the reference's published benchmark
 * (benchmark_hpc/spl_hubbard1d_bench_init.py:24-118): L sites on a ring, Jordan-Wigner
 * encoded, H = sum over bonds of h = -J (|01><10| + |10><01|) + g |11><11|; terms = the even
 * bonds (pairs (0,1), (2,3), ...) and the odd bonds ((1,2), ..., (L-1,0)); nsteps steps of
 * Suzuki's order-`order` rule over time t, neighbouring layers of one term merged.  Each
 * layer is one matchgate exp(-i tau h) (center exp(i tau J X), corner diag(1, e^{-i tau g}))
 * on all L/2 pairs of its permutation.  Writes the layers when capacity suffices and returns
 * their count (< 0 on bad arguments).
 */
static int spinless_build(int L, double J, double g, double t, int nsteps, int order, rule_t* r)
{
	if (L < 4 || L > 30 || L % 2 || nsteps < 1 || order < 2 || order % 2 || order > 12)
	{
		mg_set_error("spinless Hubbard brickwall: need an even 4 <= L <= 30, nsteps >= 1 and an even order 2..12");
		return MG_ERR_ARG;
	}
	const double h = t / nsteps;
	for (int s = 0; s < nsteps; s++)
		if (suzuki(r, order / 2, h, 2)) return -1;
	return 0;
}

int mg_spinless_hubbard_brickwall(int L, double J, double g, double t, int nsteps, int order,
	struct matchgate ulist[], int perms[], int capacity)
{
	rule_t r = { 0 };
	int rc = spinless_build(L, J, g, t, nsteps, order, &r);
	if (!rc && ulist && perms && capacity >= r.n)
		for (int l = 0; l < r.n; l++)
		{
			const double tau = r.coeff[l], c = cos(J * tau), sn = sin(J * tau);
			ulist[l] = mk(c, I * sn, I * sn, c, 1, 0, 0, cexp(-I * g * tau));
			for (int q = 0; q < L; q++) perms[l * L + q] = r.term[l] == 0 ? q : (q + 1) % L;
		}
	if (!rc) rc = r.n;
	free(r.term); free(r.coeff);
	return rc;
}

void* mg_target_spinless_hubbard(int L, double J, double g, double t, int nsteps, int order)
{
	const int n = mg_spinless_hubbard_brickwall(L, J, g, t, nsteps, order, NULL, NULL, 0);
	if (n < 0) return NULL;
	struct matchgate* u = malloc(sizeof(struct matchgate) * n);
	int* pm = malloc(sizeof(int) * (size_t)n * L);
	const int** rows = malloc(sizeof(int*) * n);
	void* h = NULL;
	if (u && pm && rows && mg_spinless_hubbard_brickwall(L, J, g, t, nsteps, order, u, pm, n) == n)
	{
		for (int l = 0; l < n; l++) rows[l] = pm + (size_t)l * L;
		h = mg_target_brickwall(u, n, rows, L);
	}
	else if (!(u && pm && rows)) mg_set_error("spinless Hubbard brickwall: out of host memory");
	free(u); free(pm); free(rows);
	return h;
}
