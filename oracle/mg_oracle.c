/*
 * ORACLE -- test infrastructure only (see mg_oracle.h).
 *
 * Restatement of the reference algorithm in this project's own code.  Citations
 * (file:line) point into the reference project rqcopt_hpc-matchgate.
 */
#include "mg_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

typedef long idx_t;

/* insert a zero bit at position p of t */
static inline idx_t ins0(idx_t t, int p)
{
	const idx_t lo = t & (((idx_t)1 << p) - 1);
	return ((t >> p) << (p + 1)) | lo;
}

/* base index of the t-th quartet for a gate on bit positions pa, pb (any order) */
static inline idx_t quartet_base(idx_t t, int pa, int pb)
{
	const int lo = pa < pb ? pa : pb, hi = pa < pb ? pb : pa;
	return ins0(ins0(t, lo), hi);
}

static void* xmalloc(size_t n)
{
	void* p = malloc(n > 0 ? n : 1);
	if (!p) { fprintf(stderr, "oracle: out of memory (%zu bytes)\n", n); abort(); }
	return p;
}

/* =====================================================================================
 * single-gate kernels
 * ===================================================================================== */

/* Apply gate g on wires (i, j) out of place; restates src/gate.c:581-652.  The
 * reference handles j < i by permuting the center block (src/gate.c:588-603); here
 * the local index is always 2*bit_i + bit_j, which gives the same products. */
void orc_apply_gate(const orc_mg* g, int i, int j, int L, const orc_c* psi, orc_c* out)
{
	const int pi = L - 1 - i, pj = L - 1 - j;
	const idx_t bi = (idx_t)1 << pi, bj = (idx_t)1 << pj;
	const idx_t nq = (idx_t)1 << (L - 2);
	for (idx_t t = 0; t < nq; t++)
	{
		const idx_t a = quartet_base(t, pi, pj);
		const orc_c x = psi[a], y = psi[a | bj], z = psi[a | bi], w = psi[a | bi | bj];
		out[a]           = g->k[0] * x + g->k[1] * w;
		out[a | bj]      = g->c[0] * y + g->c[1] * z;
		out[a | bi]      = g->c[2] * y + g->c[3] * z;
		out[a | bi | bj] = g->k[2] * x + g->k[3] * w;
	}
}

/* Backward pass of one gate: dpsi = G^T dpsi_out (no conjugation) and the gate
 * gradient as the outer product of dpsi_out and psi; restates src/gate.c:659-772. */
void orc_apply_gate_backward(const orc_mg* g, int i, int j, int L, const orc_c* psi, const orc_c* dpsi_out, orc_c* dpsi, orc_mg* dg)
{
	const int pi = L - 1 - i, pj = L - 1 - j;
	const idx_t bi = (idx_t)1 << pi, bj = (idx_t)1 << pj;
	const idx_t nq = (idx_t)1 << (L - 2);
	memset(dg, 0, sizeof(*dg));
	for (idx_t t = 0; t < nq; t++)
	{
		const idx_t a = quartet_base(t, pi, pj);
		const orc_c x = psi[a], y = psi[a | bj], z = psi[a | bi], w = psi[a | bi | bj];
		const orc_c dx = dpsi_out[a], dy = dpsi_out[a | bj], dz = dpsi_out[a | bi], dw = dpsi_out[a | bi | bj];
		dg->k[0] += dx * x; dg->k[1] += dx * w;
		dg->c[0] += dy * y; dg->c[1] += dy * z;
		dg->c[2] += dz * y; dg->c[3] += dz * z;
		dg->k[2] += dw * x; dg->k[3] += dw * w;
		dpsi[a]           = g->k[0] * dx + g->k[2] * dw;
		dpsi[a | bj]      = g->c[0] * dy + g->c[2] * dz;
		dpsi[a | bi]      = g->c[1] * dy + g->c[3] * dz;
		dpsi[a | bi | bj] = g->k[1] * dx + g->k[3] * dw;
	}
}

/* Gate applied to an interleaved array psi[2^L][nstates]; restates src/gate.c:779-851. */
void orc_apply_gate_array(const orc_mg* g, int i, int j, int L, int nstates, const orc_c* psi, orc_c* out)
{
	const int pi = L - 1 - i, pj = L - 1 - j;
	const idx_t bi = (idx_t)1 << pi, bj = (idx_t)1 << pj;
	const idx_t nq = (idx_t)1 << (L - 2);
	for (idx_t t = 0; t < nq; t++)
	{
		const idx_t a = quartet_base(t, pi, pj);
		for (int s = 0; s < nstates; s++)
		{
			const orc_c x = psi[a * nstates + s], y = psi[(a | bj) * nstates + s];
			const orc_c z = psi[(a | bi) * nstates + s], w = psi[(a | bi | bj) * nstates + s];
			out[a * nstates + s]             = g->k[0] * x + g->k[1] * w;
			out[(a | bj) * nstates + s]      = g->c[0] * y + g->c[1] * z;
			out[(a | bi) * nstates + s]      = g->c[2] * y + g->c[3] * z;
			out[(a | bi | bj) * nstates + s] = g->k[2] * x + g->k[3] * w;
		}
	}
}

/* Gate gradients of an interleaved array against one upstream derivative;
 * restates src/gate.c:858-973. */
void orc_apply_gate_backward_array(const orc_mg* g, int i, int j, int L, int nstates, const orc_c* psi, const orc_c* dpsi_out, orc_mg* dgs)
{
	(void)g;
	const int pi = L - 1 - i, pj = L - 1 - j;
	const idx_t bi = (idx_t)1 << pi, bj = (idx_t)1 << pj;
	const idx_t nq = (idx_t)1 << (L - 2);
	memset(dgs, 0, (size_t)nstates * sizeof(orc_mg));
	for (idx_t t = 0; t < nq; t++)
	{
		const idx_t a = quartet_base(t, pi, pj);
		const orc_c dx = dpsi_out[a], dy = dpsi_out[a | bj], dz = dpsi_out[a | bi], dw = dpsi_out[a | bi | bj];
		for (int s = 0; s < nstates; s++)
		{
			const orc_c x = psi[a * nstates + s], y = psi[(a | bj) * nstates + s];
			const orc_c z = psi[(a | bi) * nstates + s], w = psi[(a | bi | bj) * nstates + s];
			orc_mg* d = &dgs[s];
			d->k[0] += dx * x; d->k[1] += dx * w;
			d->c[0] += dy * y; d->c[1] += dy * z;
			d->c[2] += dz * y; d->c[3] += dz * z;
			d->k[2] += dw * x; d->k[3] += dw * w;
		}
	}
}

/* Placeholder expansion: out8[a][e] = d(G psi)[a] / dG_e for the 8 block entries
 * e = 0..3 (center) and 4..7 (corner); restates src/gate.c:982-1057. */
void orc_apply_placeholder(int i, int j, int L, const orc_c* psi, orc_c* out8)
{
	const int pi = L - 1 - i, pj = L - 1 - j;
	const idx_t bi = (idx_t)1 << pi, bj = (idx_t)1 << pj;
	const idx_t nq = (idx_t)1 << (L - 2);
	memset(out8, 0, ((size_t)1 << L) * 8 * sizeof(orc_c));
	for (idx_t t = 0; t < nq; t++)
	{
		const idx_t a = quartet_base(t, pi, pj);
		const idx_t ay = a | bj, az = a | bi, aw = a | bi | bj;
		const orc_c x = psi[a], y = psi[ay], z = psi[az], w = psi[aw];
		out8[ay * 8 + 0] = y;   /* center (0,0): out|01> += c0 y */
		out8[ay * 8 + 1] = z;   /* center (0,1) */
		out8[az * 8 + 2] = y;   /* center (1,0) */
		out8[az * 8 + 3] = z;   /* center (1,1) */
		out8[a  * 8 + 4] = x;   /* corner (0,0): out|00> += k0 x */
		out8[a  * 8 + 5] = w;   /* corner (0,1) */
		out8[aw * 8 + 6] = x;   /* corner (1,0) */
		out8[aw * 8 + 7] = w;   /* corner (1,1) */
	}
}

/* =====================================================================================
 * brickwall and general circuits
 * ===================================================================================== */

/* Brickwall: layer l applies vlist[l] to the pairs (perms[l][2p], perms[l][2p+1]);
 * restates src/matchgate_brickwall.c:14-43 (ping-pong between two buffers). */
void orc_brickwall_apply(const orc_mg* vlist, int nlayers, const int* perms, int L, const orc_c* psi, orc_c* out)
{
	const idx_t n = (idx_t)1 << L;
	orc_c* tmp = xmalloc((size_t)n * sizeof(orc_c));
	const int ng = nlayers * (L / 2);
	int k = 0;
	for (int l = 0; l < nlayers; l++)
		for (int p = 0; p < L; p += 2)
		{
			/* the final gate lands in 'out' whatever the parity of ng */
			const orc_c* src = (k == 0) ? psi : (((ng - k) % 2 == 0) ? out : tmp);
			orc_c* dst = ((ng - k) % 2 == 0) ? tmp : out;
			orc_apply_gate(&vlist[l], perms[l * L + p], perms[l * L + p + 1], L, src, dst);
			k++;
		}
	free(tmp);
}

/* Forward sweep storing the input state of every gate; src/matchgate_brickwall.c:52-78. */
void orc_brickwall_forward(const orc_mg* vlist, int nlayers, const int* perms, int L, const orc_c* psi, orc_c* cache, orc_c* out)
{
	const idx_t n = (idx_t)1 << L;
	const int ng = nlayers * (L / 2);
	memcpy(cache, psi, (size_t)n * sizeof(orc_c));
	int k = 0;
	for (int l = 0; l < nlayers; l++)
		for (int p = 0; p < L; p += 2)
		{
			orc_c* dst = (k + 1 < ng) ? cache + (k + 1) * n : out;
			orc_apply_gate(&vlist[l], perms[l * L + p], perms[l * L + p + 1], L, cache + k * n, dst);
			k++;
		}
}

/* Backward sweep summing the gate gradients per layer; src/matchgate_brickwall.c:87-127. */
void orc_brickwall_backward(const orc_mg* vlist, int nlayers, const int* perms, int L, const orc_c* cache, const orc_c* dpsi_out, orc_c* dpsi, orc_mg* dvlist)
{
	const idx_t n = (idx_t)1 << L;
	orc_c* a = xmalloc((size_t)n * sizeof(orc_c));
	orc_c* b = xmalloc((size_t)n * sizeof(orc_c));
	memcpy(a, dpsi_out, (size_t)n * sizeof(orc_c));
	int k = nlayers * (L / 2) - 1;
	for (int l = nlayers - 1; l >= 0; l--)
	{
		memset(&dvlist[l], 0, sizeof(orc_mg));
		for (int p = L - 2; p >= 0; p -= 2)
		{
			orc_mg dg;
			orc_apply_gate_backward(&vlist[l], perms[l * L + p], perms[l * L + p + 1], L, cache + k * n, a, b, &dg);
			for (int e = 0; e < 4; e++) { dvlist[l].c[e] += dg.c[e]; dvlist[l].k[e] += dg.k[e]; }
			orc_c* s = a; a = b; b = s;
			k--;
		}
	}
	memcpy(dpsi, a, (size_t)n * sizeof(orc_c));
	free(a); free(b);
}

/* add one 8x8 block h[x] (rows x = placeholder entry, columns = later-gate entry)
 * into hess at block (bi, bj) of an (nb*8)^2 matrix, scaled by mult */
static void add_block(orc_c* hess, int nb, int bi, int bj, const orc_mg* h, double mult)
{
	for (int x = 0; x < 8; x++)
		for (int y = 0; y < 4; y++)
		{
			hess[((idx_t)(bi * 8 + x) * nb + bj) * 8 + y]     += mult * h[x].c[y];
			hess[((idx_t)(bi * 8 + x) * nb + bj) * 8 + y + 4] += mult * h[x].k[y];
		}
}

/* Diagonal blocks A -> A + A^T, lower blocks mirrored from upper ones;
 * restates src/matchgate_brickwall.c:233-252. */
static void symmetrize_blocks(orc_c* hess, int nb)
{
	for (int i = 0; i < nb; i++)
		for (int x = 0; x < 8; x++)
			for (int y = 0; y <= x; y++)
			{
				const idx_t p = ((idx_t)(i * 8 + x) * nb + i) * 8 + y, q = ((idx_t)(i * 8 + y) * nb + i) * 8 + x;
				const orc_c s = hess[p] + hess[q];
				hess[p] = s; hess[q] = s;
			}
	for (int i = 0; i < nb; i++)
		for (int j = 0; j < i; j++)
			for (int x = 0; x < 8; x++)
				for (int y = 0; y < 8; y++)
					hess[((idx_t)(i * 8 + x) * nb + j) * 8 + y] = hess[((idx_t)(j * 8 + y) * nb + i) * 8 + x];
}

/* Backward sweep with a cache of upstream derivatives, then the Hessian from
 * placeholder states pushed through all later gates; restates
 * src/matchgate_brickwall.c:137-260 (ti = 0) and :308-435 (ti = 1: one placement
 * per layer, weighted by the number of translated copies). */
void orc_brickwall_backward_hessian(const orc_mg* vlist, int nlayers, const int* perms, int L, int ti, const orc_c* cache,
	const orc_c* dpsi_out, orc_c* dpsi, orc_mg* dvlist, orc_c* hess)
{
	const idx_t n = (idx_t)1 << L;
	const int half = L / 2;
	const int ng = nlayers * half;
	orc_c* gcache = xmalloc((size_t)ng * n * sizeof(orc_c));

	/* gradient, keeping the derivative that enters each gate's backward step */
	memcpy(gcache + (idx_t)(ng - 1) * n, dpsi_out, (size_t)n * sizeof(orc_c));
	int k = ng - 1;
	for (int l = nlayers - 1; l >= 0; l--)
	{
		memset(&dvlist[l], 0, sizeof(orc_mg));
		for (int p = L - 2; p >= 0; p -= 2)
		{
			orc_c* dst = (k > 0) ? gcache + (idx_t)(k - 1) * n : dpsi;
			orc_mg dg;
			orc_apply_gate_backward(&vlist[l], perms[l * L + p], perms[l * L + p + 1], L, cache + (idx_t)k * n, gcache + (idx_t)k * n, dst, &dg);
			for (int e = 0; e < 4; e++) { dvlist[l].c[e] += dg.c[e]; dvlist[l].k[e] += dg.k[e]; }
			k--;
		}
	}

	const int m = nlayers * 8;
	memset(hess, 0, (size_t)m * m * sizeof(orc_c));
	orc_c* t0 = xmalloc((size_t)n * 8 * sizeof(orc_c));
	orc_c* t1 = xmalloc((size_t)n * 8 * sizeof(orc_c));
	orc_mg h[8];
	for (int i = 0; i < nlayers; i++)
	{
		const int rmax = ti ? 1 : half;
		for (int rr = 0; rr < rmax; rr++)
		{
			const int r = 2 * rr;
			const int kp = i * half + rr;   /* sequential index of the placement */
			orc_apply_placeholder(perms[i * L + r], perms[i * L + r + 1], L, cache + (idx_t)kp * n, t0);
			orc_c* cur = t0; orc_c* nxt = t1;
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
					orc_apply_gate_backward_array(&vlist[j], perms[j * L + s], perms[j * L + s + 1], L, 8, cur, gcache + (idx_t)lidx * n, h);
					add_block(hess, nlayers, i, j, h, mult);
					if (j < nlayers - 1 || s < L - 2)
					{
						orc_apply_gate_array(&vlist[j], perms[j * L + s], perms[j * L + s + 1], L, 8, cur, nxt);
						orc_c* sw = cur; cur = nxt; nxt = sw;
					}
					lidx++;
				}
			}
		}
	}
	symmetrize_blocks(hess, nlayers);
	free(t1); free(t0); free(gcache);
}

/* General circuit, gate g on wires (wires[2g], wires[2g+1]); src/quantum_circuit.c:13-35. */
void orc_circuit_apply(const orc_mg* gates, int ngates, const int* wires, int L, const orc_c* psi, orc_c* out)
{
	const idx_t n = (idx_t)1 << L;
	orc_c* tmp = xmalloc((size_t)n * sizeof(orc_c));
	for (int g = 0; g < ngates; g++)
	{
		const orc_c* src = (g == 0) ? psi : (((ngates - g) % 2 == 0) ? out : tmp);
		orc_c* dst = ((ngates - g) % 2 == 0) ? tmp : out;
		orc_apply_gate(&gates[g], wires[2 * g], wires[2 * g + 1], L, src, dst);
	}
	if (ngates == 0) memcpy(out, psi, (size_t)n * sizeof(orc_c));
	free(tmp);
}

/* src/quantum_circuit.c:90-108 */
void orc_circuit_forward(const orc_mg* gates, int ngates, const int* wires, int L, const orc_c* psi, orc_c* cache, orc_c* out)
{
	const idx_t n = (idx_t)1 << L;
	memcpy(cache, psi, (size_t)n * sizeof(orc_c));
	for (int g = 0; g < ngates; g++)
	{
		orc_c* dst = (g + 1 < ngates) ? cache + (idx_t)(g + 1) * n : out;
		orc_apply_gate(&gates[g], wires[2 * g], wires[2 * g + 1], L, cache + (idx_t)g * n, dst);
	}
}

/* Per-gate gradients; src/quantum_circuit.c:115-140. */
void orc_circuit_backward(const orc_mg* gates, int ngates, const int* wires, int L, const orc_c* cache, const orc_c* dpsi_out, orc_c* dpsi, orc_mg* dgates)
{
	const idx_t n = (idx_t)1 << L;
	orc_c* a = xmalloc((size_t)n * sizeof(orc_c));
	orc_c* b = xmalloc((size_t)n * sizeof(orc_c));
	memcpy(a, dpsi_out, (size_t)n * sizeof(orc_c));
	for (int g = ngates - 1; g >= 0; g--)
	{
		orc_apply_gate_backward(&gates[g], wires[2 * g], wires[2 * g + 1], L, cache + (idx_t)g * n, a, b, &dgates[g]);
		orc_c* s = a; a = b; b = s;
	}
	memcpy(dpsi, a, (size_t)n * sizeof(orc_c));
	free(a); free(b);
}

/* =====================================================================================
 * targets
 * ===================================================================================== */

enum { T_HASH = 0, T_DENSE = 1, T_BRICKWALL = 2, T_CIRCUIT = 3 };

struct orc_target
{
	int kind, L;
	orc_c* dense;
	orc_mg* gates;
	int* wires;
	int ngates;
};

orc_target* orc_target_hash(int L)
{
	orc_target* t = xmalloc(sizeof(*t));
	memset(t, 0, sizeof(*t));
	t->kind = T_HASH; t->L = L;
	return t;
}

orc_target* orc_target_dense(const orc_c* U, int L)
{
	orc_target* t = orc_target_hash(L);
	const size_t n = (size_t)1 << L;
	t->kind = T_DENSE;
	t->dense = xmalloc(n * n * sizeof(orc_c));
	memcpy(t->dense, U, n * n * sizeof(orc_c));
	return t;
}

/* a brickwall target is stored as the equivalent sequential circuit */
orc_target* orc_target_brickwall(const orc_mg* ulist, int ulayers, const int* uperms, int L)
{
	orc_target* t = orc_target_hash(L);
	t->kind = T_BRICKWALL;
	t->ngates = ulayers * (L / 2);
	t->gates = xmalloc((size_t)t->ngates * sizeof(orc_mg));
	t->wires = xmalloc((size_t)t->ngates * 2 * sizeof(int));
	int g = 0;
	for (int l = 0; l < ulayers; l++)
		for (int p = 0; p < L; p += 2)
		{
			t->gates[g] = ulist[l];
			t->wires[2 * g] = uperms[l * L + p];
			t->wires[2 * g + 1] = uperms[l * L + p + 1];
			g++;
		}
	return t;
}

orc_target* orc_target_circuit(const orc_mg* gates, int ngates, const int* wires, int L)
{
	orc_target* t = orc_target_hash(L);
	t->kind = T_CIRCUIT;
	t->ngates = ngates;
	t->gates = xmalloc((size_t)(ngates > 0 ? ngates : 1) * sizeof(orc_mg));
	t->wires = xmalloc((size_t)(ngates > 0 ? ngates : 1) * 2 * sizeof(int));
	memcpy(t->gates, gates, (size_t)ngates * sizeof(orc_mg));
	memcpy(t->wires, wires, (size_t)ngates * 2 * sizeof(int));
	return t;
}

void orc_target_free(orc_target* t)
{
	if (!t) return;
	free(t->dense); free(t->gates); free(t->wires); free(t);
}

/* out = U psi; scratch holds 2^L entries */
void orc_target_apply(const orc_target* t, const orc_c* psi, orc_c* out, orc_c* scratch)
{
	const idx_t n = (idx_t)1 << t->L;
	switch (t->kind)
	{
	case T_HASH:   /* test/test_matchgate_target.c:20-34 */
		for (idx_t i = 0; i < n; i++)
			out[i] = (-1.1 + 0.8 * I) * psi[((i + 3) * 113) % n] + (0.4 - 0.7 * I) * psi[((i + 9) * 173) % n]
			       + (0.5 + 0.1 * I) * psi[i] + (-0.3 + 0.2 * I) * psi[((i + 4) * 199) % n];
		break;
	case T_DENSE:  /* zgemv, test/test_matchgate_target.c:38-47 */
		for (idx_t i = 0; i < n; i++)
		{
			orc_c s = 0;
			for (idx_t j = 0; j < n; j++) s += t->dense[i * n + j] * psi[j];
			out[i] = s;
		}
		break;
	default:       /* sequential gates, ping-pong through scratch */
	{
		const int ng = t->ngates;
		if (ng == 0) { memcpy(out, psi, (size_t)n * sizeof(orc_c)); break; }
		for (int g = 0; g < ng; g++)
		{
			const orc_c* src = (g == 0) ? psi : (((ng - g) % 2 == 0) ? out : scratch);
			orc_c* dst = ((ng - g) % 2 == 0) ? scratch : out;
			orc_apply_gate(&t->gates[g], t->wires[2 * g], t->wires[2 * g + 1], t->L, src, dst);
		}
	}
	}
}

/* =====================================================================================
 * traces over basis columns
 * ===================================================================================== */

static void brickwall_to_circuit(const orc_mg* vlist, int nlayers, const int* perms, int L, orc_mg* gates, int* wires)
{
	/* src/matchgate_target.c:308-324 */
	int g = 0;
	for (int l = 0; l < nlayers; l++)
		for (int p = 0; p < L; p += 2)
		{
			gates[g] = vlist[l];
			wires[2 * g] = perms[l * L + p];
			wires[2 * g + 1] = perms[l * L + p + 1];
			g++;
		}
}

static int resolve_threads(int nthreads) { return nthreads > 0 ? nthreads : omp_get_max_threads(); }

static void col_range(int L, long* b0, long* b1)
{
	const long n = 1L << L;
	if (*b1 < 0 || *b1 > n) *b1 = n;
	if (*b0 < 0) *b0 = 0;
	if (*b0 > *b1) *b0 = *b1;
}

/* Upsi = -conj(U e_b) (src/matchgate_target.c:254-266) */
static void target_column(const orc_target* t, long b, orc_c* e, orc_c* upsi, orc_c* scratch)
{
	const idx_t n = (idx_t)1 << t->L;
	memset(e, 0, (size_t)n * sizeof(orc_c));
	e[b] = 1;
	orc_target_apply(t, e, upsi, scratch);
	for (idx_t a = 0; a < n; a++) upsi[a] = -conj(upsi[a]);
}

/* f = sum_b <-conj(U e_b), C e_b>; restates src/matchgate_target.c:20-80 and the
 * OpenMP column split of :83-203 (per-thread partial sums, combined in thread order). */
int orc_circuit_target(const orc_target* t, const orc_mg* gates, int ngates, const int* wires, int L,
	int nthreads, long b0, long b1, orc_c* fval)
{
	col_range(L, &b0, &b1);
	const int nt = resolve_threads(nthreads);
	const idx_t n = (idx_t)1 << L;
	orc_c* part = xmalloc((size_t)nt * sizeof(orc_c));
	#pragma omp parallel num_threads(nt)
	{
		const int tid = omp_get_thread_num();
		orc_c* e = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* up = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* cp = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* sc = xmalloc((size_t)n * sizeof(orc_c));
		orc_c f = 0;
		#pragma omp for schedule(static)
		for (long b = b0; b < b1; b++)
		{
			target_column(t, b, e, up, sc);
			e[b] = 1;
			orc_circuit_apply(gates, ngates, wires, L, e, cp);
			for (idx_t a = 0; a < n; a++) f += up[a] * cp[a];
		}
		part[tid] = f;
		free(sc); free(cp); free(up); free(e);
	}
	orc_c f = 0;
	for (int i = 0; i < nt; i++) f += part[i];
	free(part);
	*fval = f;
	return 0;
}

/* f and per-gate gradients; restates src/matchgate_target.c:212-302, with the
 * column loop split over threads as in the reference's parallel variants. */
int orc_circuit_target_and_gradient(const orc_target* t, const orc_mg* gates, int ngates, const int* wires, int L,
	int nthreads, long b0, long b1, orc_c* fval, orc_mg* dgates)
{
	col_range(L, &b0, &b1);
	const int nt = resolve_threads(nthreads);
	const idx_t n = (idx_t)1 << L;
	orc_c* fpart = xmalloc((size_t)nt * sizeof(orc_c));
	orc_mg* gpart = xmalloc((size_t)nt * ngates * sizeof(orc_mg));
	memset(gpart, 0, (size_t)nt * ngates * sizeof(orc_mg));
	#pragma omp parallel num_threads(nt)
	{
		const int tid = omp_get_thread_num();
		orc_c* e = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* up = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* cp = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* sc = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* cache = xmalloc((size_t)(ngates > 0 ? ngates : 1) * n * sizeof(orc_c));
		orc_mg* dg = xmalloc((size_t)(ngates > 0 ? ngates : 1) * sizeof(orc_mg));
		orc_mg* acc = &gpart[(size_t)tid * ngates];
		orc_c f = 0;
		#pragma omp for schedule(static)
		for (long b = b0; b < b1; b++)
		{
			target_column(t, b, e, up, sc);
			e[b] = 1;
			orc_circuit_forward(gates, ngates, wires, L, e, cache, cp);
			for (idx_t a = 0; a < n; a++) f += up[a] * cp[a];
			orc_circuit_backward(gates, ngates, wires, L, cache, up, e, dg);
			for (int g = 0; g < ngates; g++)
				for (int q = 0; q < 4; q++) { acc[g].c[q] += dg[g].c[q]; acc[g].k[q] += dg[g].k[q]; }
		}
		fpart[tid] = f;
		free(dg); free(cache); free(sc); free(cp); free(up); free(e);
	}
	orc_c f = 0;
	memset(dgates, 0, (size_t)ngates * sizeof(orc_mg));
	for (int i = 0; i < nt; i++)
	{
		f += fpart[i];
		for (int g = 0; g < ngates; g++)
			for (int q = 0; q < 4; q++) { dgates[g].c[q] += gpart[(size_t)i * ngates + g].c[q]; dgates[g].k[q] += gpart[(size_t)i * ngates + g].k[q]; }
	}
	free(gpart); free(fpart);
	*fval = f;
	return 0;
}

/* Per-gate Hessian (an extension: the reference has per-layer Hessians only).  The
 * same placeholder method as src/matchgate_brickwall.c:177-231 with every gate its
 * own block: hess is (8*ngates)^2, row (g*8+x), column (h*8+y), symmetric with zero
 * diagonal blocks (each gate enters the circuit linearly). */
int orc_circuit_target_gradient_hessian(const orc_target* t, const orc_mg* gates, int ngates, const int* wires, int L,
	int nthreads, long b0, long b1, orc_c* fval, orc_mg* dgates, orc_c* hess)
{
	col_range(L, &b0, &b1);
	const int nt = resolve_threads(nthreads);
	const idx_t n = (idx_t)1 << L;
	const idx_t m = 8 * (idx_t)ngates;
	orc_c* fpart = xmalloc((size_t)nt * sizeof(orc_c));
	orc_mg* gpart = xmalloc((size_t)nt * ngates * sizeof(orc_mg));
	orc_c* hpart = xmalloc((size_t)nt * m * m * sizeof(orc_c));
	memset(gpart, 0, (size_t)nt * ngates * sizeof(orc_mg));
	memset(hpart, 0, (size_t)nt * m * m * sizeof(orc_c));
	#pragma omp parallel num_threads(nt)
	{
		const int tid = omp_get_thread_num();
		orc_c* e = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* up = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* cp = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* sc = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* cache = xmalloc((size_t)ngates * n * sizeof(orc_c));
		orc_c* gcache = xmalloc((size_t)ngates * n * sizeof(orc_c));
		orc_c* t0 = xmalloc((size_t)n * 8 * sizeof(orc_c));
		orc_c* t1 = xmalloc((size_t)n * 8 * sizeof(orc_c));
		orc_mg* acc = &gpart[(size_t)tid * ngates];
		orc_c* hacc = &hpart[(size_t)tid * m * m];
		orc_mg h[8];
		orc_c f = 0;
		#pragma omp for schedule(static)
		for (long b = b0; b < b1; b++)
		{
			target_column(t, b, e, up, sc);
			e[b] = 1;
			orc_circuit_forward(gates, ngates, wires, L, e, cache, cp);
			for (idx_t a = 0; a < n; a++) f += up[a] * cp[a];
			memcpy(gcache + (idx_t)(ngates - 1) * n, up, (size_t)n * sizeof(orc_c));
			for (int g = ngates - 1; g >= 0; g--)
			{
				orc_c* dst = (g > 0) ? gcache + (idx_t)(g - 1) * n : e;
				orc_mg dg;
				orc_apply_gate_backward(&gates[g], wires[2 * g], wires[2 * g + 1], L, cache + (idx_t)g * n, gcache + (idx_t)g * n, dst, &dg);
				for (int q = 0; q < 4; q++) { acc[g].c[q] += dg.c[q]; acc[g].k[q] += dg.k[q]; }
			}
			for (int g = 0; g < ngates; g++)
			{
				orc_apply_placeholder(wires[2 * g], wires[2 * g + 1], L, cache + (idx_t)g * n, t0);
				orc_c* cur = t0; orc_c* nxt = t1;
				for (int l = g + 1; l < ngates; l++)
				{
					orc_apply_gate_backward_array(&gates[l], wires[2 * l], wires[2 * l + 1], L, 8, cur, gcache + (idx_t)l * n, h);
					for (int x = 0; x < 8; x++)
						for (int y = 0; y < 4; y++)
						{
							hacc[(g * 8 + x) * m + l * 8 + y]     += h[x].c[y];
							hacc[(g * 8 + x) * m + l * 8 + y + 4] += h[x].k[y];
						}
					if (l < ngates - 1)
					{
						orc_apply_gate_array(&gates[l], wires[2 * l], wires[2 * l + 1], L, 8, cur, nxt);
						orc_c* sw = cur; cur = nxt; nxt = sw;
					}
				}
			}
		}
		fpart[tid] = f;
		free(t1); free(t0); free(gcache); free(cache); free(sc); free(cp); free(up); free(e);
	}
	orc_c f = 0;
	memset(dgates, 0, (size_t)ngates * sizeof(orc_mg));
	memset(hess, 0, (size_t)m * m * sizeof(orc_c));
	for (int i = 0; i < nt; i++)
	{
		f += fpart[i];
		for (int g = 0; g < ngates; g++)
			for (int q = 0; q < 4; q++) { dgates[g].c[q] += gpart[(size_t)i * ngates + g].c[q]; dgates[g].k[q] += gpart[(size_t)i * ngates + g].k[q]; }
		for (idx_t q = 0; q < m * m; q++) hess[q] += hpart[(size_t)i * m * m + q];
	}
	/* mirror the upper block triangle into the lower one */
	for (idx_t r = 0; r < m; r++)
		for (idx_t c = 0; c < m; c++)
			if (c / 8 < r / 8) hess[r * m + c] = hess[c * m + r];
	free(hpart); free(gpart); free(fpart);
	*fval = f;
	return 0;
}

/* src/matchgate_target.c:333-350 */
int orc_brickwall_target(const orc_target* t, const orc_mg* vlist, int nlayers, const int* perms, int L,
	int nthreads, long b0, long b1, orc_c* fval)
{
	const int ng = nlayers * (L / 2);
	orc_mg* gates = xmalloc((size_t)ng * sizeof(orc_mg));
	int* wires = xmalloc((size_t)ng * 2 * sizeof(int));
	brickwall_to_circuit(vlist, nlayers, perms, L, gates, wires);
	int ret = orc_circuit_target(t, gates, ng, wires, L, nthreads, b0, b1, fval);
	free(wires); free(gates);
	return ret;
}

/* src/matchgate_target.c:359-388: per-gate gradients summed per layer */
int orc_brickwall_target_and_gradient(const orc_target* t, const orc_mg* vlist, int nlayers, const int* perms, int L,
	int nthreads, long b0, long b1, orc_c* fval, orc_mg* dvlist)
{
	const int half = L / 2, ng = nlayers * half;
	orc_mg* gates = xmalloc((size_t)ng * sizeof(orc_mg));
	orc_mg* dg = xmalloc((size_t)ng * sizeof(orc_mg));
	int* wires = xmalloc((size_t)ng * 2 * sizeof(int));
	brickwall_to_circuit(vlist, nlayers, perms, L, gates, wires);
	int ret = orc_circuit_target_and_gradient(t, gates, ng, wires, L, nthreads, b0, b1, fval, dg);
	for (int l = 0; l < nlayers; l++)
	{
		memset(&dvlist[l], 0, sizeof(orc_mg));
		for (int p = 0; p < half; p++)
			for (int q = 0; q < 4; q++) { dvlist[l].c[q] += dg[l * half + p].c[q]; dvlist[l].k[q] += dg[l * half + p].k[q]; }
	}
	free(wires); free(dg); free(gates);
	return ret;
}

/* Column loop with forward cache, overlap and the backward/Hessian sweep; restates
 * src/matchgate_target.c:397-513 (plain), :515-624 (ti) and :626-869 (threads). */
int orc_brickwall_target_gradient_hessian(const orc_target* t, const orc_mg* vlist, int nlayers, const int* perms, int L, int ti,
	int nthreads, long b0, long b1, orc_c* fval, orc_mg* dvlist, orc_c* hess)
{
	col_range(L, &b0, &b1);
	const int nt = resolve_threads(nthreads);
	const idx_t n = (idx_t)1 << L;
	const int ng = nlayers * (L / 2);
	const idx_t m = 8 * (idx_t)nlayers;
	orc_c* fpart = xmalloc((size_t)nt * sizeof(orc_c));
	orc_mg* gpart = xmalloc((size_t)nt * nlayers * sizeof(orc_mg));
	orc_c* hpart = xmalloc((size_t)nt * m * m * sizeof(orc_c));
	memset(gpart, 0, (size_t)nt * nlayers * sizeof(orc_mg));
	memset(hpart, 0, (size_t)nt * m * m * sizeof(orc_c));
	#pragma omp parallel num_threads(nt)
	{
		const int tid = omp_get_thread_num();
		orc_c* e = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* up = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* wp = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* sc = xmalloc((size_t)n * sizeof(orc_c));
		orc_c* cache = xmalloc((size_t)ng * n * sizeof(orc_c));
		orc_mg* dv = xmalloc((size_t)nlayers * sizeof(orc_mg));
		orc_c* hu = xmalloc((size_t)m * m * sizeof(orc_c));
		orc_c f = 0;
		#pragma omp for schedule(static)
		for (long b = b0; b < b1; b++)
		{
			target_column(t, b, e, up, sc);
			e[b] = 1;
			orc_brickwall_forward(vlist, nlayers, perms, L, e, cache, wp);
			for (idx_t a = 0; a < n; a++) f += up[a] * wp[a];
			orc_brickwall_backward_hessian(vlist, nlayers, perms, L, ti, cache, up, e, dv, hu);
			for (int l = 0; l < nlayers; l++)
				for (int q = 0; q < 4; q++) { gpart[(size_t)tid * nlayers + l].c[q] += dv[l].c[q]; gpart[(size_t)tid * nlayers + l].k[q] += dv[l].k[q]; }
			for (idx_t q = 0; q < m * m; q++) hpart[(size_t)tid * m * m + q] += hu[q];
		}
		fpart[tid] = f;
		free(hu); free(dv); free(cache); free(sc); free(wp); free(up); free(e);
	}
	orc_c f = 0;
	memset(dvlist, 0, (size_t)nlayers * sizeof(orc_mg));
	memset(hess, 0, (size_t)m * m * sizeof(orc_c));
	for (int i = 0; i < nt; i++)
	{
		f += fpart[i];
		for (int l = 0; l < nlayers; l++)
			for (int q = 0; q < 4; q++) { dvlist[l].c[q] += gpart[(size_t)i * nlayers + l].c[q]; dvlist[l].k[q] += gpart[(size_t)i * nlayers + l].k[q]; }
		for (idx_t q = 0; q < m * m; q++) hess[q] += hpart[(size_t)i * m * m + q];
	}
	free(hpart); free(gpart); free(fpart);
	*fval = f;
	return 0;
}

/* Riemannian gradient vector: conj then tangent-to-real per layer
 * (src/matchgate_target.c:903-908) applied to the brickwall gradient. */
int orc_brickwall_projected_gradient(const orc_target* t, const orc_mg* vlist, int nlayers, const int* perms, int L,
	int nthreads, long b0, long b1, orc_c* fval, double* grad_vec)
{
	orc_mg* dv = xmalloc((size_t)nlayers * sizeof(orc_mg));
	int ret = orc_brickwall_target_and_gradient(t, vlist, nlayers, perms, L, nthreads, b0, b1, fval, dv);
	for (int l = 0; l < nlayers; l++)
	{
		orc_mg_conj(&dv[l]);
		orc_mg_tangent_to_real(&vlist[l], &dv[l], &grad_vec[l * 8]);
	}
	free(dv);
	return ret;
}

/* =====================================================================================
 * matchgate algebra (src/matchgate.c)
 * ===================================================================================== */

static void mat2_mul(const orc_c* a, const orc_c* b, orc_c* c)
{
	/* src/matchgate.c:338-352 (accumulation order kept) */
	orc_c r[4] = { 0, 0, 0, 0 };
	for (int i = 0; i < 2; i++)
		for (int j = 0; j < 2; j++)
			for (int k = 0; k < 2; k++)
				r[2 * i + k] += a[2 * i + j] * b[2 * j + k];
	memcpy(c, r, sizeof(r));
}

void orc_mg_multiply(const orc_mg* a, const orc_mg* b, orc_mg* c)
{
	orc_mg r;
	mat2_mul(a->c, b->c, r.c);
	mat2_mul(a->k, b->k, r.k);
	*c = r;
}

void orc_mg_adjoint(const orc_mg* a, orc_mg* ah)
{
	orc_mg r;
	for (int i = 0; i < 2; i++)
		for (int j = 0; j < 2; j++) { r.c[2 * i + j] = conj(a->c[2 * j + i]); r.k[2 * i + j] = conj(a->k[2 * j + i]); }
	*ah = r;
}

void orc_mg_conj(orc_mg* a)
{
	for (int q = 0; q < 4; q++) { a->c[q] = conj(a->c[q]); a->k[q] = conj(a->k[q]); }
}

/* Hermitian part per block; src/matchgate.c:196-212 */
void orc_mg_symm(const orc_mg* w, orc_mg* z)
{
	orc_mg r;
	r.k[0] = creal(w->k[0]); r.c[0] = creal(w->c[0]); r.c[3] = creal(w->c[3]); r.k[3] = creal(w->k[3]);
	r.k[1] = 0.5 * (w->k[1] + conj(w->k[2]));
	r.c[1] = 0.5 * (w->c[1] + conj(w->c[2]));
	r.k[2] = conj(r.k[1]);
	r.c[2] = conj(r.c[1]);
	*z = r;
}

/* anti-Hermitian part per block; src/matchgate.c:219-243 */
void orc_mg_antisymm(const orc_mg* w, orc_mg* z)
{
	orc_mg r;
	r.k[0] = I * cimag(w->k[0]); r.c[0] = I * cimag(w->c[0]); r.c[3] = I * cimag(w->c[3]); r.k[3] = I * cimag(w->k[3]);
	r.k[1] = 0.5 * (w->k[1] - conj(w->k[2]));
	r.c[1] = 0.5 * (w->c[1] - conj(w->c[2]));
	r.k[2] = -conj(r.k[1]);
	r.c[2] = -conj(r.c[1]);
	*z = r;
}

/* 8 reals -> anti-Hermitian U(2)+U(2) tangent; src/matchgate.c:251-270 */
void orc_mg_real_to_antisymm(const double* r, orc_mg* w)
{
	w->c[0] = I * r[0];
	w->c[3] = I * r[3];
	w->k[0] = I * r[4];
	w->k[3] = I * r[7];
	w->c[1] = 0.5 * (r[1] - r[2]) + 0.5 * I * (r[1] + r[2]);
	w->k[1] = 0.5 * (r[5] - r[6]) + 0.5 * I * (r[5] + r[6]);
	w->c[2] = -conj(w->c[1]);
	w->k[2] = -conj(w->k[1]);
}

/* src/matchgate.c:277-288 */
void orc_mg_antisymm_to_real(const orc_mg* w, double* r)
{
	for (int q = 0; q < 4; q++)
	{
		r[q]     = creal(w->c[q]) + cimag(w->c[q]);
		r[q + 4] = creal(w->k[q]) + cimag(w->k[q]);
	}
}

/* src/matchgate.c:296-301 */
void orc_mg_real_to_tangent(const double* r, const orc_mg* v, orc_mg* z)
{
	orc_mg a;
	orc_mg_real_to_antisymm(r, &a);
	orc_mg_multiply(v, &a, z);
}

/* src/matchgate.c:309-316 */
void orc_mg_tangent_to_real(const orc_mg* v, const orc_mg* z, double* r)
{
	orc_mg w, t;
	orc_mg_adjoint(v, &w);
	orc_mg_multiply(&w, z, &t);
	orc_mg_antisymm(&t, &w);
	orc_mg_antisymm_to_real(&w, r);
}

/* p = z - u symm(u^H z); src/matchgate.c:323-334 */
void orc_mg_project_tangent(const orc_mg* u, const orc_mg* z, orc_mg* p)
{
	orc_mg v, w;
	orc_mg_adjoint(u, &v);
	orc_mg_multiply(&v, z, &w);
	orc_mg_symm(&w, &v);
	orc_mg_multiply(u, &v, &w);
	for (int q = 0; q < 4; q++) { p->c[q] = z->c[q] - w.c[q]; p->k[q] = z->k[q] - w.k[q]; }
}

/* (a b c + c b a) / 2; src/matchgate.c:381-393 */
static void sym_triple(const orc_mg* a, const orc_mg* b, const orc_mg* c, orc_mg* ret)
{
	orc_mg u, v;
	orc_mg_multiply(a, b, &u);
	orc_mg_multiply(&u, c, ret);
	orc_mg_multiply(c, b, &u);
	orc_mg_multiply(&u, a, &v);
	for (int q = 0; q < 4; q++) { ret->c[q] = 0.5 * (ret->c[q] + v.c[q]); ret->k[q] = 0.5 * (ret->k[q] + v.k[q]); }
}

/* 2x2 inverse by Gauss-Jordan elimination with partial pivoting; src/matchgate.c:414-479 */
static int mat2_inv(const orc_c* a, orc_c* out)
{
	orc_c m[4] = { a[0], a[1], a[2], a[3] };
	orc_c v[4] = { 1, 0, 0, 1 };
	for (int k = 0; k < 2; k++)
	{
		int piv = k;
		double p = cabs(m[2 * k + k]);
		if (k == 0 && cabs(m[2]) > p) { piv = 1; p = cabs(m[2]); }
		if (p == 0) return -1;
		if (piv != k)
			for (int c = 0; c < 2; c++)
			{
				orc_c s = m[2 * k + c]; m[2 * k + c] = m[2 * piv + c]; m[2 * piv + c] = s;
				s = v[2 * k + c]; v[2 * k + c] = v[2 * piv + c]; v[2 * piv + c] = s;
			}
		const int o = 1 - k;
		const orc_c f = m[2 * o + k] / m[2 * k + k];
		for (int c = k + 1; c < 2; c++) m[2 * o + c] -= f * m[2 * k + c];
		m[2 * o + k] = 0;
		for (int c = 0; c < 2; c++) v[2 * o + c] -= f * v[2 * k + c];
		for (int c = k + 1; c < 2; c++) m[2 * k + c] /= m[2 * k + k];
		for (int c = 0; c < 2; c++) v[2 * k + c] /= m[2 * k + k];
		m[2 * k + k] = 1;
	}
	memcpy(out, v, sizeof(v));
	return 0;
}

int orc_mg_inverse(const orc_mg* a, orc_mg* ainv)
{
	orc_mg r;
	int e = mat2_inv(a->c, r.c) | mat2_inv(a->k, r.k);
	*ainv = r;
	return e ? -1 : 0;
}

static double unif_dist4(const orc_c* a, const orc_c* b)
{
	double d = 0;
	for (int q = 0; q < 4; q++) d = fmax(d, cabs(a[q] - b[q]));
	return d;
}

/* Newton iteration u <- (u + u^{-H}) / 2 per block; src/matchgate.c:517-541 */
void orc_mg_polar(const orc_mg* a, orc_mg* u)
{
	orc_mg cur = *a;
	for (int it = 0; it < 14; it++)
	{
		orc_mg inv, w;
		orc_mg_inverse(&cur, &inv);
		orc_mg_adjoint(&inv, &w);
		for (int q = 0; q < 4; q++) { cur.c[q] = 0.5 * (cur.c[q] + w.c[q]); cur.k[q] = 0.5 * (cur.k[q] + w.k[q]); }
		if (it >= 4 && unif_dist4(cur.c, w.c) < 1e-14 && unif_dist4(cur.k, w.k) < 1e-14) break;
	}
	*u = cur;
}

/* v = polar(u (I + A(eta))); src/matchgate.c:548-562 */
void orc_mg_retract(const orc_mg* u, const double* eta, orc_mg* v)
{
	orc_mg z, w;
	orc_mg_real_to_antisymm(eta, &z);
	z.k[0] += 1; z.c[0] += 1; z.c[3] += 1; z.k[3] += 1;
	orc_mg_multiply(u, &z, &w);
	orc_mg_polar(&w, v);
}

/* Real Riemannian Hessian from the complex one; restates src/matchgate_target.c:910-967.
 * dvlist_conj holds the already conjugated gate gradients. */
void orc_project_hessian(const orc_mg* vlist, const orc_mg* dvc, int nlayers, const orc_c* hess, double* H)
{
	const int m = 8 * nlayers;
	for (int i = 0; i < nlayers; i++)
		for (int j = i; j < nlayers; j++)
			for (int k = 0; k < 8; k++)
			{
				double r[8] = { 0 };
				r[k] = 1;
				orc_mg Z, G;
				orc_mg_real_to_tangent(r, &vlist[j], &Z);
				memset(&G, 0, sizeof(G));
				for (int x = 0; x < 4; x++)
					for (int y = 0; y < 4; y++)
					{
						G.c[x] += hess[((i * 8 + x) * nlayers + j) * 8 + y] * Z.c[y] + hess[((i * 8 + x) * nlayers + j) * 8 + y + 4] * Z.k[y];
						G.k[x] += hess[((i * 8 + x + 4) * nlayers + j) * 8 + y] * Z.c[y] + hess[((i * 8 + x + 4) * nlayers + j) * 8 + y + 4] * Z.k[y];
					}
				orc_mg_conj(&G);
				if (i == j)
				{
					orc_mg P, gh, T;
					orc_mg_project_tangent(&vlist[i], &G, &P);
					orc_mg_adjoint(&dvc[i], &gh);
					sym_triple(&Z, &gh, &vlist[i], &T);
					for (int q = 0; q < 4; q++) { G.c[q] = P.c[q] - T.c[q]; G.k[q] = P.k[q] - T.k[q]; }
				}
				orc_mg_tangent_to_real(&vlist[i], &G, r);
				for (int x = 0; x < 8; x++) H[((i * 8 + x) * nlayers + j) * 8 + k] = r[x];
			}
	for (int i = 0; i < m; i++)
		for (int j = 0; j < i; j++) H[i * m + j] = H[j * m + i];
}

/* src/matchgate_target.c:877-973 */
int orc_brickwall_gradvec_hessmat(const orc_target* t, const orc_mg* vlist, int nlayers, const int* perms, int L, int ti,
	int nthreads, orc_c* fval, double* grad_vec, double* H)
{
	const int m = 8 * nlayers;
	orc_mg* dv = xmalloc((size_t)nlayers * sizeof(orc_mg));
	orc_c* hess = xmalloc((size_t)m * m * sizeof(orc_c));
	int ret = orc_brickwall_target_gradient_hessian(t, vlist, nlayers, perms, L, ti, nthreads, 0, -1, fval, dv, hess);
	for (int l = 0; l < nlayers; l++)
	{
		orc_mg_conj(&dv[l]);
		orc_mg_tangent_to_real(&vlist[l], &dv[l], &grad_vec[l * 8]);
	}
	orc_project_hessian(vlist, dv, nlayers, hess, H);
	free(hess); free(dv);
	return ret;
}

/* =====================================================================================
 * trust region (src/trust_region.c)
 * ===================================================================================== */

static double dot(const double* a, const double* b, int n)
{
	double s = 0;
	for (int i = 0; i < n; i++) s += a[i] * b[i];
	return s;
}

/* t > 0 with ||b + t d|| = radius; src/trust_region.c:17-74 */
static double to_boundary(const double* b, const double* d, int n, double radius)
{
	const double dd = dot(d, d, n);
	if (dd == 0) return 0;
	const double p = dot(b, d, n) / dd;
	const double q = (dot(b, b, n) - radius * radius) / dd;
	if (p == 0) return sqrt(-q);
	const double a = -(p + copysign(1.0, p) * sqrt(p * p - q));
	const double c = q / a;
	return a <= c ? c : a;
}

/* Steihaug truncated CG on an explicit Hessian; src/trust_region.c:88-146.
 * Returns 1 when the step stopped on the trust-region boundary. */
int orc_truncated_cg(const double* grad, const double* hess, int n, double radius, int maxiter, double abstol, double reltol, double* z)
{
	double* r = xmalloc((size_t)n * sizeof(double));
	double* d = xmalloc((size_t)n * sizeof(double));
	double* hd = xmalloc((size_t)n * sizeof(double));
	memcpy(r, grad, (size_t)n * sizeof(double));
	double rsq = dot(r, r, n);
	const double stoptol = fmax(abstol, reltol * sqrt(rsq));
	memset(z, 0, (size_t)n * sizeof(double));
	for (int i = 0; i < n; i++) d[i] = -r[i];
	int boundary = 0;
	for (int it = 0; it < maxiter; it++)
	{
		for (int i = 0; i < n; i++) hd[i] = dot(&hess[(size_t)i * n], d, n);
		const double dhd = dot(d, hd, n);
		const double tb = to_boundary(z, d, n, radius);
		const double alpha = rsq / dhd;
		if (dhd <= 0 || alpha > tb)
		{
			for (int i = 0; i < n; i++) z[i] += tb * d[i];
			boundary = 1;
			break;
		}
		for (int i = 0; i < n; i++) r[i] += alpha * hd[i];
		for (int i = 0; i < n; i++) z[i] += alpha * d[i];
		const double rsq1 = dot(r, r, n);
		if (sqrt(rsq1) <= stoptol) break;
		const double beta = rsq1 / rsq;
		for (int i = 0; i < n; i++) d[i] = beta * d[i] - r[i];
		rsq = rsq1;
	}
	free(hd); free(d); free(r);
	return boundary;
}

/* Riemannian trust region over the brickwall gates (Absil et al., Alg. 10);
 * restates src/trust_region.c:235-306 driven as in src/mg_brickwall_opt.c:99-122. */
void orc_rtr_brickwall(const orc_target* t, const orc_mg* vlist0, int nlayers, const int* perms, int L, int ti, int nthreads,
	int niter, int tcg_maxiter, double rho_trust, double radius_init, double maxradius,
	double* f_iter, orc_c* f_citer, orc_mg* vlist_out)
{
	const int n = 8 * nlayers;
	orc_mg* x = xmalloc((size_t)nlayers * sizeof(orc_mg));
	orc_mg* xn = xmalloc((size_t)nlayers * sizeof(orc_mg));
	double* grad = xmalloc((size_t)n * sizeof(double));
	double* hess = xmalloc((size_t)n * n * sizeof(double));
	double* eta = xmalloc((size_t)n * sizeof(double));
	double* heta = xmalloc((size_t)n * sizeof(double));
	memcpy(x, vlist0, (size_t)nlayers * sizeof(orc_mg));
	double radius = radius_init;
	for (int it = 0; it < niter; it++)
	{
		orc_c fc;
		orc_brickwall_gradvec_hessmat(t, x, nlayers, perms, L, ti, nthreads, &fc, grad, hess);
		const double fx = creal(fc);
		const int onb = orc_truncated_cg(grad, hess, n, radius, tcg_maxiter, 1e-8, 1e-6, eta);
		for (int l = 0; l < nlayers; l++) orc_mg_retract(&x[l], &eta[l * 8], &xn[l]);
		f_iter[it] = fx;
		f_citer[it] = fc;
		for (int i = 0; i < n; i++) heta[i] = dot(&hess[(size_t)i * n], eta, n);
		orc_c fn;
		orc_brickwall_target(t, xn, nlayers, perms, L, nthreads, 0, -1, &fn);
		const double rho = (creal(fn) - fx) / (dot(grad, eta, n) + 0.5 * dot(eta, heta, n));
		if (rho < 0.25) radius *= 0.25;
		else if (rho > 0.75 && onb) radius = fmin(2 * radius, maxradius);
		if (rho > rho_trust) { orc_mg* s = x; x = xn; xn = s; }
	}
	memcpy(vlist_out, x, (size_t)nlayers * sizeof(orc_mg));
	orc_c ff;
	orc_brickwall_target(t, x, nlayers, perms, L, nthreads, 0, -1, &ff);
	f_iter[niter] = creal(ff);
	f_citer[niter] = ff;
	free(heta); free(eta); free(hess); free(grad); free(xn); free(x);
}
