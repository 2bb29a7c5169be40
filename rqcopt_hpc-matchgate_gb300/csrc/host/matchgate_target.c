/*
 * Target function, gradients and Hessians as traces over basis columns (reference
 * src/matchgate_target.c), evaluated by the batched GPU engine.  This file turns the
 * reference's calls into evaluation plans, keeps recent plans for reuse (a trust-region
 * run calls the same shapes over and over), and implements the GPU target handles and
 * the device-resident plan API of mg_gb300.h.
 */
#include <stdint.h>
#include <stdio.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "matchgate_target.h"
#include "mg_gb300.h"
#include "../mg_internal.h"
#include "mg_host.h"

/* ======================================================================================
 * GPU target handles
 * ====================================================================================== */

static mg_target_handle* as_handle(linear_func f, void* udata)
{
	if (f != mg_target_apply || !udata) return NULL;
	mg_target_handle* h = (mg_target_handle*)udata;
	return h->magic == MG_TARGET_MAGIC ? h : NULL;
}

int mg_target_apply(const struct statevector* restrict psi, void* udata, struct statevector* restrict psi_out)
{
	mg_target_handle* h = (mg_target_handle*)udata;
	if (!h || h->magic != MG_TARGET_MAGIC || psi->nqubits != h->L || psi_out->nqubits != h->L)
	{
		mg_set_error("mg_target_apply: invalid target handle or qubit count");
		return -1;
	}
	mgcu_lock();
	int r = mgcu_target_apply(h->dev, (const mgc*)psi->data, (mgc*)psi_out->data);
	mgcu_unlock();
	return r ? -1 : 0;
}

static void* wrap_target(mgcu_target* t, int L)
{
	if (!t) return NULL;
	mg_target_handle* h = malloc(sizeof(*h));
	if (!h) { mgcu_target_destroy(t); return NULL; }
	h->magic = MG_TARGET_MAGIC; h->L = L; h->dev = t;
	return h;
}

void* mg_target_circuit(const struct matchgate gates[], int ngates, const int wires[], int nqubits)
{
	for (int g = 0; g < 2 * ngates; g++)
		if (wires[g] < 0 || wires[g] >= nqubits || (g % 2 && wires[g] == wires[g - 1]))
		{
			mg_set_error("mg_target_circuit: invalid wires of gate %d", g / 2);
			return NULL;
		}
	mgcu_lock();
	void* h = wrap_target(mgcu_target_circuit((const mgg*)gates, wires, ngates, nqubits), nqubits);
	mgcu_unlock();
	return h;
}

void* mg_target_brickwall(const struct matchgate ulist[], int ulayers, const int* uperms[], int nqubits)
{
	const int half = nqubits / 2, ng = ulayers * half;
	struct matchgate* g = malloc(sizeof(*g) * (ng > 0 ? ng : 1));
	int* w = malloc(sizeof(int) * 2 * (ng > 0 ? ng : 1));
	if (!g || !w) { free(g); free(w); return NULL; }
	for (int i = 0; i < ulayers; i++)
		for (int p = 0; p < half; p++)
		{
			g[i * half + p] = ulist[i];
			w[2 * (i * half + p)] = uperms[i][2 * p];
			w[2 * (i * half + p) + 1] = uperms[i][2 * p + 1];
		}
	void* h = mg_target_circuit(g, ng, w, nqubits);
	free(g); free(w);
	return h;
}

void* mg_target_dense(const numeric* U, int nqubits)
{
	mgcu_lock();
	void* h = wrap_target(mgcu_target_dense((const mgc*)U, nqubits), nqubits);
	mgcu_unlock();
	return h;
}

static void plan_cache_drop_target(mgcu_target* t);

void mg_target_free(void* udata)
{
	mg_target_handle* h = (mg_target_handle*)udata;
	if (!h || h->magic != MG_TARGET_MAGIC) return;
	mgcu_lock();
	plan_cache_drop_target(h->dev);
	mgcu_target_destroy(h->dev);
	mgcu_unlock();
	h->magic = 0;
	free(h);
}

int mg_target_set_resident(void* udata, int enable)
{
	mg_target_handle* h = (mg_target_handle*)udata;
	if (!h || h->magic != MG_TARGET_MAGIC) { mg_set_error("mg_target_set_resident: invalid handle"); return MG_ERR_ARG; }
	mgcu_lock();
	mgcu_target_set_resident(h->dev, enable);
	mgcu_unlock();
	return 0;
}

int mgh_target_resident(void* udata)
{
	mg_target_handle* h = (mg_target_handle*)udata;
	if (!h || h->magic != MG_TARGET_MAGIC) return -1;
	mgcu_lock();
	const int r = mgcu_target_resident(h->dev);
	mgcu_unlock();
	return r;
}

int mg_target_conserves_weight(void* udata)
{
	mg_target_handle* h = (mg_target_handle*)udata;
	if (!h || h->magic != MG_TARGET_MAGIC) { mg_set_error("mg_target_conserves_weight: invalid handle"); return -1; }
	mgcu_lock();
	const int n = mgcu_target_conserves_weight(h->dev);
	mgcu_unlock();
	return n;
}

int mg_target_sweep_gates(void* udata)
{
	mg_target_handle* h = (mg_target_handle*)udata;
	if (!h || h->magic != MG_TARGET_MAGIC) { mg_set_error("mg_target_sweep_gates: invalid handle"); return -1; }
	mgcu_lock();
	const int n = mgcu_target_sweep_gates(h->dev);
	mgcu_unlock();
	return n;
}

/* ======================================================================================
 * plan cache
 * ====================================================================================== */
typedef struct
{
	uint64_t hash;
	int L, ngates, nblocks, want_grad, want_hess, ti, precision;
	long opts[MG_NOPTIONS + 1];
	mgcu_target* target;
	int* wires;
	int* block;
	mgcu_plan* plan;
	unsigned long stamp;
} plan_entry;

#define PLAN_CACHE 16
static plan_entry g_plans[PLAN_CACHE];
static unsigned long g_stamp;

static uint64_t fnv(uint64_t h, const void* p, size_t n)
{
	const unsigned char* c = (const unsigned char*)p;
	for (size_t i = 0; i < n; i++) { h ^= c[i]; h *= 1099511628211ull; }
	return h;
}

static void entry_free(plan_entry* e)
{
	if (e->plan) mgcu_plan_destroy(e->plan);
	free(e->wires); free(e->block);
	memset(e, 0, sizeof(*e));
}

static void plan_cache_drop_target(mgcu_target* t)
{
	for (int i = 0; i < PLAN_CACHE; i++)
		if (g_plans[i].plan && g_plans[i].target == t) entry_free(&g_plans[i]);
}

/* Hessian placements and weights.  Plain: every gate is a placement, every later gate
 * has weight 1 (src/matchgate_brickwall.c:177-231).  Translation invariant: only the
 * first pair of each layer, weighted by the number of translated copies, L/2, less the
 * pair offset inside the placement's own layer (src/matchgate_brickwall.c:363-404). */
static int make_placements(int ngates, int half, int ti, int** place, double** w, int* nplace)
{
	const int np = ti ? ngates / half : ngates;
	*place = malloc(sizeof(int) * (np > 0 ? np : 1));
	*w = calloc((size_t)(np > 0 ? np : 1) * (ngates > 0 ? ngates : 1), sizeof(double));
	if (!*place || !*w) { free(*place); free(*w); return -1; }
	for (int p = 0; p < np; p++)
	{
		const int k = ti ? p * half : p;
		(*place)[p] = k;
		for (int l = k + 1; l < ngates; l++)
		{
			double m = 1.0;
			if (ti)
			{
				m = half;
				if (l / half == k / half) m -= (l - k);
			}
			(*w)[(size_t)p * ngates + l] = m;
		}
	}
	*nplace = np;
	return 0;
}

static mgcu_plan* get_plan(int L, int ngates, const int* wires, int nblocks, const int* block, int want_grad, int want_hess, int ti,
	mgcu_target* target)
{
	const int prec = mgcu_precision();
	long opts[MG_NOPTIONS + 1];
	for (int o = 1; o <= MG_NOPTIONS; o++) opts[o] = mgcu_option(o);
	opts[0] = 0;
	uint64_t h = 1469598103934665603ull;
	h = fnv(h, wires, sizeof(int) * 2 * ngates);
	h = fnv(h, block, sizeof(int) * ngates);
	for (int i = 0; i < PLAN_CACHE; i++)
	{
		plan_entry* e = &g_plans[i];
		if (e->plan && e->hash == h && e->L == L && e->ngates == ngates && e->nblocks == nblocks && e->want_grad == want_grad &&
			e->want_hess == want_hess && e->ti == ti && e->precision == prec && e->target == target &&
			!memcmp(e->opts, opts, sizeof(opts)) && !memcmp(e->wires, wires, sizeof(int) * 2 * ngates) &&
			!memcmp(e->block, block, sizeof(int) * ngates))
		{
			e->stamp = ++g_stamp;
			return e->plan;
		}
	}
	mgcu_plan_desc d;
	memset(&d, 0, sizeof(d));
	d.L = L; d.ngates = ngates; d.wires = wires; d.nblocks = nblocks; d.block = block;
	d.want_grad = want_grad; d.want_hess = want_hess; d.target = target; d.precision = prec;
	int* place = NULL;
	double* w = NULL;
	if (want_hess)
	{
		if (make_placements(ngates, L / 2, ti, &place, &w, &d.nplace)) return NULL;
		d.place = place; d.place_w = w;
	}
	mgcu_plan* p = mgcu_plan_create(&d);
	free(place); free(w);
	if (!p) return NULL;
	/* evict the least recently used entry */
	int slot = 0;
	for (int i = 0; i < PLAN_CACHE; i++)
	{
		if (!g_plans[i].plan) { slot = i; break; }
		if (g_plans[i].stamp < g_plans[slot].stamp) slot = i;
	}
	entry_free(&g_plans[slot]);
	plan_entry* e = &g_plans[slot];
	e->hash = h; e->L = L; e->ngates = ngates; e->nblocks = nblocks; e->want_grad = want_grad; e->want_hess = want_hess;
	e->ti = ti; e->precision = prec; e->target = target; e->plan = p; e->stamp = ++g_stamp;
	memcpy(e->opts, opts, sizeof(opts));
	e->wires = malloc(sizeof(int) * 2 * (ngates > 0 ? ngates : 1));
	e->block = malloc(sizeof(int) * (ngates > 0 ? ngates : 1));
	if (!e->wires || !e->block) { entry_free(e); return NULL; }
	memcpy(e->wires, wires, sizeof(int) * 2 * ngates);
	memcpy(e->block, block, sizeof(int) * ngates);
	return p;
}

/* ======================================================================================
 * evaluation driver
 * ====================================================================================== */

/* -conj(U e_b) on b's parity sector for b in [c0, c1), from a host linear_func.  The caller's
 * map is called from several host threads at once, as the reference calls it from its
 * OpenMP threads (src/matchgate_target.c:788-795); each thread owns its input and output
 * vectors and the columns b = c0 + tid (mod nthreads), so the result does not depend on
 * the thread count. */
typedef struct
{
	linear_func ufunc;
	void* udata;
	int L, nthreads, tid;
	long c0, c1;
	mgc* cols;
	int* failed;     /* shared: set by the first failing call, stops the others */
	int rc;          /* this thread's result */
} mat_job;

static void* mat_worker(void* arg)
{
	mat_job* j = (mat_job*)arg;
	const long n = 1L << j->L, S = n >> 1;
	struct statevector psi, out;
	j->rc = 0;
	if (allocate_statevector(j->L, &psi) < 0) { j->rc = MG_ERR_ALLOC; __atomic_store_n(j->failed, 1, __ATOMIC_RELAXED); return NULL; }
	if (allocate_statevector(j->L, &out) < 0)
	{
		free_statevector(&psi);
		j->rc = MG_ERR_ALLOC;
		__atomic_store_n(j->failed, 1, __ATOMIC_RELAXED);
		return NULL;
	}
	memset(psi.data, 0, sizeof(numeric) * n);
	for (long b = j->c0 + j->tid; b < j->c1; b += j->nthreads)
	{
		if (__atomic_load_n(j->failed, __ATOMIC_RELAXED)) break;
		psi.data[b] = 1;
		const int ret = j->ufunc(&psi, j->udata, &out);
		psi.data[b] = 0;
		if (ret < 0)
		{
			fprintf(stderr, "call of 'ufunc' failed, return value: %i\n", ret);
			mg_set_error("call of 'ufunc' failed, return value: %i", ret);
			j->rc = MG_ERR_UFUNC;
			__atomic_store_n(j->failed, 1, __ATOMIC_RELAXED);
			break;
		}
		const int pb = __builtin_popcountl(b) & 1;
		mgc* col = j->cols + (size_t)(b - j->c0) * S;
		for (long c = 0; c < S; c++)
		{
			const long a = (c << 1) | ((__builtin_popcountl(c) + pb) & 1);
			col[c] = mgc_make(-creal(out.data[a]), cimag(out.data[a]));
		}
	}
	free_statevector(&out);
	free_statevector(&psi);
	return NULL;
}

/* host threads for a host map: MG_OPT_HOST_THREADS, else the online cores */
static int host_threads(long ncols)
{
	long t = mgcu_option(MG_OPT_HOST_THREADS_ID);
	if (t <= 0) t = sysconf(_SC_NPROCESSORS_ONLN);
	if (t < 1) t = 1;
	if (t > 256) t = 256;
	if (t > ncols) t = ncols;
	return (int)t;
}

static int materialise(linear_func ufunc, void* udata, int L, long c0, long c1, mgc* cols)
{
	if (c1 <= c0) return 0;
	const int nt = host_threads(c1 - c0);
	int failed = 0;
	mat_job* jobs = calloc((size_t)nt, sizeof(mat_job));
	pthread_t* th = calloc((size_t)nt, sizeof(pthread_t));
	if (!jobs || !th) { free(jobs); free(th); return MG_ERR_ALLOC; }
	int started = 0;
	for (int t = 0; t < nt; t++)
	{
		jobs[t] = (mat_job){ ufunc, udata, L, nt, t, c0, c1, cols, &failed, 0 };
		if (t == 0) continue;   /* the calling thread takes share 0 */
		if (pthread_create(&th[t], NULL, mat_worker, &jobs[t]) != 0) { jobs[t].rc = MG_ERR_ALLOC; failed = 1; break; }
		started = t;
	}
	if (!failed) mat_worker(&jobs[0]);
	for (int t = 1; t <= started; t++) pthread_join(th[t], NULL);
	int rc = 0;
	for (int t = 0; t < nt && !rc; t++) rc = jobs[t].rc;
	free(jobs);
	free(th);
	return rc;
}

typedef struct
{
	int L, ngates, nblocks;
	const struct matchgate* gates;   /* [ngates] */
	const int* wires;                /* [2 ngates] */
	const int* block;                /* [ngates] */
	int want_grad, want_hess, ti;
	long b0, b1;
	/* outputs (any may be NULL) */
	numeric* fval;
	struct matchgate* dblocks;       /* [nblocks] */
	numeric* hess;                   /* [(8 nblocks)^2] */
	const struct matchgate* vblocks; /* gates per block, for the projections */
	double* grad_vec;
	double* H;
} eval_req;

static int run_eval(linear_func ufunc, void* udata, const eval_req* q)
{
	if (q->L < 3)
	{
		mg_set_error("the batched evaluation needs at least 3 qubits (got %d)", q->L);
		return MG_ERR_ARG;
	}
	mg_target_handle* th = as_handle(ufunc, udata);
	if (th && th->L != q->L)
	{
		mg_set_error("target has %d qubits, circuit has %d", th->L, q->L);
		return MG_ERR_ARG;
	}
	const long ncols = 1L << q->L;
	const long b0 = q->b0 < 0 ? 0 : q->b0;
	const long b1 = (q->b1 < 0 || q->b1 > ncols) ? ncols : q->b1;
	mgcu_lock();
	int rc = 0;
	mgcu_plan* p = get_plan(q->L, q->ngates, q->wires, q->nblocks, q->block, q->want_grad, q->want_hess, q->ti, th ? th->dev : NULL);
	if (!p) rc = MG_ERR_DEVICE;
	if (!rc) rc = mgcu_plan_set_gates(p, (const mgg*)q->gates);
	if (!rc) rc = mgcu_plan_begin(p);
	if (!rc)
	{
		if (th) rc = mgcu_plan_columns(p, b0, b1, NULL);
		else
		{
			/* chunks of at most 1/8 of the range (at least 1024 columns): the caller's map fills
			 * chunk k + 1 on the host threads while the GPU works on chunk k (the copy of a
			 * chunk from this pageable buffer completes before its call returns) */
			long chunk = mgcu_plan_chunk_columns(p);
			const long part = (b1 - b0 + 7) / 8 > 1024 ? (b1 - b0 + 7) / 8 : 1024;
			if (chunk > part) chunk = part;
			const long S = ncols >> 1;
			mgc* cols = malloc(sizeof(mgc) * S * (size_t)(chunk < b1 - b0 ? chunk : b1 - b0 > 0 ? b1 - b0 : 1));
			if (!cols) rc = MG_ERR_ALLOC;
			for (long c0 = b0; c0 < b1 && !rc; c0 += chunk)
			{
				const long c1 = c0 + chunk < b1 ? c0 + chunk : b1;
				mgcu_unlock();   /* the caller's map may itself use this library */
				rc = materialise(ufunc, udata, q->L, c0, c1, cols);
				mgcu_lock();
				if (!rc) rc = mgcu_plan_columns(p, c0, c1, cols);
			}
			free(cols);
		}
	}
	if (!rc) rc = mgcu_plan_finish(p);
	mgc f;
	if (!rc) rc = mgcu_plan_fetch(p, &f, (mgg*)q->dblocks, (mgc*)q->hess);
	if (!rc && (q->grad_vec || q->H)) rc = mgcu_plan_project(p, (const mgg*)q->vblocks, q->grad_vec, q->H);
	mgcu_unlock();
	if (rc)
	{
		if (rc != MG_ERR_UFUNC) fprintf(stderr, "matchgate evaluation failed (code %d): %s\n", rc, mg_last_error());
		return rc;
	}
	if (q->fval) *q->fval = f.re + I * f.im;
	return 0;
}

/* brickwall -> sequential circuit with one block per layer (src/matchgate_target.c:308-324) */
int brickwall_seq(const struct matchgate vlist[], int nlayers, int L, const int* perms[], seq_circuit* s)
{
	if (L % 2 || nlayers < 1)
	{
		mg_set_error("a brickwall needs an even number of qubits and at least one layer");
		return MG_ERR_ARG;
	}
	const int half = L / 2, ng = nlayers * half;
	s->ngates = ng;
	s->gates = malloc(sizeof(struct matchgate) * ng);
	s->wires = malloc(sizeof(int) * 2 * ng);
	s->block = malloc(sizeof(int) * ng);
	if (!s->gates || !s->wires || !s->block) { free(s->gates); free(s->wires); free(s->block); return MG_ERR_ALLOC; }
	for (int i = 0; i < nlayers; i++)
		for (int p = 0; p < half; p++)
		{
			const int g = i * half + p;
			s->gates[g] = vlist[i];
			s->wires[2 * g] = perms[i][2 * p];
			s->wires[2 * g + 1] = perms[i][2 * p + 1];
			s->block[g] = i;
		}
	return 0;
}

void seq_free(seq_circuit* s) { free(s->gates); free(s->wires); free(s->block); }

static int* identity_blocks(int n)
{
	int* b = malloc(sizeof(int) * (n > 0 ? n : 1));
	if (b) for (int i = 0; i < n; i++) b[i] = i;
	return b;
}

/* the translation-invariant Hessian in place of the plain one: the reference's build flag
 * TRANSLATIONAL_INVARIANCE (src/matchgate_target.c:478,715,819) as a runtime option */
static int ti_build(void) { return mgcu_option(MG_OPT_TRANSLATIONAL_INVARIANCE_ID) != 0; }

static int brickwall_eval(linear_func ufunc, void* udata, const struct matchgate vlist[], int nlayers, int L, const int* perms[],
	int want_grad, int want_hess, int ti, long b0, long b1, numeric* fval, struct matchgate* dvlist, numeric* hess, double* grad_vec, double* H)
{
	seq_circuit s;
	int rc = brickwall_seq(vlist, nlayers, L, perms, &s);
	if (rc) return rc;
	eval_req q;
	memset(&q, 0, sizeof(q));
	q.L = L; q.ngates = s.ngates; q.nblocks = nlayers; q.gates = s.gates; q.wires = s.wires; q.block = s.block;
	q.want_grad = want_grad; q.want_hess = want_hess; q.ti = ti; q.b0 = b0; q.b1 = b1;
	q.fval = fval; q.dblocks = dvlist; q.hess = hess; q.vblocks = vlist; q.grad_vec = grad_vec; q.H = H;
	rc = run_eval(ufunc, udata, &q);
	seq_free(&s);
	return rc;
}

static int circuit_eval(linear_func ufunc, void* udata, const struct matchgate gates[], int ngates, const int wires[], int L,
	int want_grad, int want_hess, numeric* fval, struct matchgate* dgates, numeric* hess, double* grad_vec, double* H)
{
	int* blk = identity_blocks(ngates);
	if (!blk) return MG_ERR_ALLOC;
	eval_req q;
	memset(&q, 0, sizeof(q));
	q.L = L; q.ngates = ngates; q.nblocks = ngates; q.gates = gates; q.wires = wires; q.block = blk;
	q.want_grad = want_grad; q.want_hess = want_hess; q.b0 = 0; q.b1 = -1;
	q.fval = fval; q.dblocks = dgates; q.hess = hess; q.vblocks = gates; q.grad_vec = grad_vec; q.H = H;
	int rc = run_eval(ufunc, udata, &q);
	free(blk);
	return rc;
}

/* ======================================================================================
 * reference entry points
 * ====================================================================================== */

int matchgate_circuit_unitary_target(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits, numeric* fval)
{
	return circuit_eval(ufunc, udata, gates, ngates, wires, nqubits, 0, 0, fval, NULL, NULL, NULL, NULL);
}

int parallel_matchgate_circuit_unitary_target(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits, numeric* fval)
{
	return matchgate_circuit_unitary_target(ufunc, udata, gates, ngates, wires, nqubits, fval);
}

int matchgate_circuit_unitary_target_and_gradient(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits,
	numeric* fval, struct matchgate dgates[])
{
	return circuit_eval(ufunc, udata, gates, ngates, wires, nqubits, 1, 0, fval, dgates, NULL, NULL, NULL);
}

int matchgate_circuit_unitary_target_gradient_hessian(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits,
	numeric* fval, struct matchgate dgates[], numeric* hess)
{
	return circuit_eval(ufunc, udata, gates, ngates, wires, nqubits, 1, 1, fval, dgates, hess, NULL, NULL);
}

/* per-gate Riemannian forms: the projection of src/matchgate_target.c:877-973 with one
 * parameter block per gate instead of per layer */
int matchgate_circuit_unitary_target_and_projected_gradient(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits,
	numeric* fval, double* grad_vec)
{
	return circuit_eval(ufunc, udata, gates, ngates, wires, nqubits, 1, 0, fval, NULL, NULL, grad_vec, NULL);
}

int matchgate_circuit_unitary_target_gradient_vector_hessian_matrix(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits,
	numeric* fval, double* grad_vec, double* H)
{
	return circuit_eval(ufunc, udata, gates, ngates, wires, nqubits, 1, 1, fval, NULL, NULL, grad_vec, H);
}

int matchgate_brickwall_unitary_target(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[], numeric* fval)
{
	return brickwall_eval(ufunc, udata, vlist, nlayers, nqubits, perms, 0, 0, 0, 0, -1, fval, NULL, NULL, NULL, NULL);
}

int matchgate_brickwall_unitary_target_and_gradient(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, struct matchgate dvlist[])
{
	return brickwall_eval(ufunc, udata, vlist, nlayers, nqubits, perms, 1, 0, 0, 0, -1, fval, dvlist, NULL, NULL, NULL);
}

int mg_brickwall_target_and_gradient_columns(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	long col_begin, long col_end, numeric* fval, struct matchgate dvlist[])
{
	if (col_begin < 0 || col_end < col_begin || col_end > (1L << nqubits))
	{
		mg_set_error("column range [%ld, %ld) outside [0, 2^%d)", col_begin, col_end, nqubits);
		return MG_ERR_ARG;
	}
	return brickwall_eval(ufunc, udata, vlist, nlayers, nqubits, perms, dvlist != NULL, 0, 0, col_begin, col_end, fval, dvlist, NULL, NULL, NULL);
}

int matchgate_brickwall_unitary_target_gradient_hessian(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, struct matchgate dvlist[], numeric* hess)
{
	return brickwall_eval(ufunc, udata, vlist, nlayers, nqubits, perms, 1, 1, ti_build(), 0, -1, fval, dvlist, hess, NULL, NULL);
}

int matchgate_ti_brickwall_unitary_target_gradient_hessian(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, struct matchgate dvlist[], numeric* hess)
{
	return brickwall_eval(ufunc, udata, vlist, nlayers, nqubits, perms, 1, 1, 1, 0, -1, fval, dvlist, hess, NULL, NULL);
}

int parallel_matchgate_brickwall_unitary_target_gradient_hessian(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, struct matchgate dvlist[], numeric* hess)
{
	return matchgate_brickwall_unitary_target_gradient_hessian(ufunc, udata, vlist, nlayers, nqubits, perms, fval, dvlist, hess);
}

int matchgate_brickwall_unitary_target_gradient_vector_hessian_matrix(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, double* grad_vec, double* H)
{
	return brickwall_eval(ufunc, udata, vlist, nlayers, nqubits, perms, 1, 1, ti_build(), 0, -1, fval, NULL, NULL, grad_vec, H);
}

int matchgate_brickwall_unitary_target_and_projected_gradient(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, double* grad_vec)
{
	return brickwall_eval(ufunc, udata, vlist, nlayers, nqubits, perms, 1, 0, 0, 0, -1, fval, NULL, NULL, grad_vec, NULL);
}

/* ======================================================================================
 * device-resident plans
 * ====================================================================================== */
struct mg_plan
{
	mgcu_plan* p;
	seq_circuit s;
	int nlayers, L;             /* nlayers: parameter blocks (layers, or gates of a circuit plan) */
	int circuit;                /* 1: one block per gate (mg_plan_circuit) */
	struct matchgate* vlist;
};

mg_plan* mg_plan_brickwall(linear_func ufunc, void* udata, const struct matchgate vlist[], int nlayers, int nqubits,
	const int* perms[], int what)
{
	mg_target_handle* th = as_handle(ufunc, udata);
	if (!th || th->L != nqubits)
	{
		mg_set_error("mg_plan_brickwall needs a GPU target (mg_target_*) on the same qubits");
		return NULL;
	}
	mg_plan* pl = calloc(1, sizeof(*pl));
	if (!pl) return NULL;
	if (brickwall_seq(vlist, nlayers, nqubits, perms, &pl->s)) { free(pl); return NULL; }
	pl->nlayers = nlayers; pl->L = nqubits;
	pl->vlist = malloc(sizeof(struct matchgate) * nlayers);
	mgcu_plan_desc d;
	memset(&d, 0, sizeof(d));
	d.L = nqubits; d.ngates = pl->s.ngates; d.wires = pl->s.wires; d.nblocks = nlayers; d.block = pl->s.block;
	d.want_grad = (what & 3) >= MG_EVAL_GRADIENT; d.want_hess = (what & 3) == MG_EVAL_HESSIAN;
	d.target = th->dev; d.precision = mgcu_precision();
	int* place = NULL;
	double* w = NULL;
	if (d.want_hess && make_placements(d.ngates, nqubits / 2, (what & MG_EVAL_TI) != 0, &place, &w, &d.nplace)) { mg_plan_free(pl); return NULL; }
	d.place = place; d.place_w = w;
	mgcu_lock();
	pl->p = mgcu_plan_create(&d);
	mgcu_unlock();
	free(place); free(w);
	if (!pl->p || !pl->vlist || mg_plan_set_gates(pl, vlist)) { mg_plan_free(pl); return NULL; }
	return pl;
}

mg_plan* mg_plan_circuit(linear_func ufunc, void* udata, const struct matchgate gates[], int ngates, const int wires[],
	int nqubits, int what)
{
	mg_target_handle* th = as_handle(ufunc, udata);
	if (!th || th->L != nqubits)
	{
		mg_set_error("mg_plan_circuit needs a GPU target (mg_target_*) on the same qubits");
		return NULL;
	}
	if (ngates < 1 || (what & MG_EVAL_TI))
	{
		mg_set_error("mg_plan_circuit: needs at least one gate; the translation-invariant Hessian is for brickwalls");
		return NULL;
	}
	mg_plan* pl = calloc(1, sizeof(*pl));
	if (!pl) return NULL;
	pl->circuit = 1;
	pl->nlayers = ngates; pl->L = nqubits;
	pl->s.ngates = ngates;
	pl->s.gates = malloc(sizeof(struct matchgate) * ngates);
	pl->s.wires = malloc(sizeof(int) * 2 * ngates);
	pl->s.block = identity_blocks(ngates);
	pl->vlist = malloc(sizeof(struct matchgate) * ngates);
	if (!pl->s.gates || !pl->s.wires || !pl->s.block || !pl->vlist) { mg_plan_free(pl); return NULL; }
	memcpy(pl->s.wires, wires, sizeof(int) * 2 * ngates);
	mgcu_plan_desc d;
	memset(&d, 0, sizeof(d));
	d.L = nqubits; d.ngates = ngates; d.wires = pl->s.wires; d.nblocks = ngates; d.block = pl->s.block;
	d.want_grad = (what & 3) >= MG_EVAL_GRADIENT; d.want_hess = (what & 3) == MG_EVAL_HESSIAN;
	d.target = th->dev; d.precision = mgcu_precision();
	int* place = NULL;
	double* w = NULL;
	if (d.want_hess && make_placements(ngates, nqubits / 2, 0, &place, &w, &d.nplace)) { mg_plan_free(pl); return NULL; }
	d.place = place; d.place_w = w;
	mgcu_lock();
	pl->p = mgcu_plan_create(&d);
	mgcu_unlock();
	free(place); free(w);
	if (!pl->p || mg_plan_set_gates(pl, gates)) { mg_plan_free(pl); return NULL; }
	return pl;
}

int mg_plan_set_gates(mg_plan* pl, const struct matchgate vlist[])
{
	const int half = pl->L / 2;
	memcpy(pl->vlist, vlist, sizeof(struct matchgate) * pl->nlayers);
	if (pl->circuit) memcpy(pl->s.gates, vlist, sizeof(struct matchgate) * pl->nlayers);
	else
		for (int i = 0; i < pl->nlayers; i++)
			for (int p = 0; p < half; p++) pl->s.gates[i * half + p] = vlist[i];
	mgcu_lock();
	int r = mgcu_plan_set_gates(pl->p, (const mgg*)pl->s.gates);
	mgcu_unlock();
	return r;
}

int mg_plan_run(mg_plan* pl)
{
	mgcu_lock();
	int r = mgcu_plan_begin(pl->p);
	if (!r) r = mgcu_plan_columns(pl->p, 0, 1L << pl->L, NULL);
	if (!r) r = mgcu_plan_finish(pl->p);
	mgcu_unlock();
	return r;
}

int mg_plan_results(mg_plan* pl, numeric* fval, struct matchgate dvlist[], numeric* hess, double* grad_vec, double* H)
{
	mgcu_lock();
	mgc f;
	int r = mgcu_plan_fetch(pl->p, &f, (mgg*)dvlist, (mgc*)hess);
	if (!r && (grad_vec || H)) r = mgcu_plan_project(pl->p, (const mgg*)pl->vlist, grad_vec, H);
	mgcu_unlock();
	if (!r && fval) *fval = f.re + I * f.im;
	return r;
}

void mg_plan_free(mg_plan* pl)
{
	if (!pl) return;
	mgcu_lock();
	if (pl->p) mgcu_plan_destroy(pl->p);
	mgcu_unlock();
	seq_free(&pl->s);
	free(pl->vlist);
	free(pl);
}

double mg_plan_time_ms(mg_plan* pl, int steps, int flush_l2)
{
	mgcu_lock();
	double r = mgcu_plan_time_ms(pl->p, 0, 1L << pl->L, steps, flush_l2);
	mgcu_unlock();
	return r;
}

int mg_plan_target_kernel_ms(mg_plan* pl, double* ms, long* launches)
{
	if (!pl || !ms || !launches) { mg_set_error("mg_plan_target_kernel_ms: null argument"); return MG_ERR_ARG; }
	mgcu_lock();
	const int e = mgcu_plan_target_kernel_ms(pl->p, ms, launches);
	mgcu_unlock();
	return e ? MG_ERR_DEVICE : 0;
}

int mg_plan_target_config(const mg_plan* pl, int cfg[4])
{
	if (!pl || !cfg) { mg_set_error("mg_plan_target_config: null argument"); return MG_ERR_ARG; }
	mgcu_plan_target_config(pl->p, cfg);
	return 0;
}

/* ======================================================================================
 * batches
 * ====================================================================================== */
struct mg_batch
{
	mgcu_batch* b;
	int n;
	int* nlayers;
	int* L;
	seq_circuit* s;
	struct matchgate** vlist;
};

void mg_batch_free(mg_batch* bt)
{
	if (!bt) return;
	if (bt->b) { mgcu_lock(); mgcu_batch_destroy(bt->b); mgcu_unlock(); }
	for (int i = 0; i < bt->n; i++)
	{
		if (bt->s) seq_free(&bt->s[i]);
		if (bt->vlist) free(bt->vlist[i]);
	}
	free(bt->s); free(bt->vlist); free(bt->nlayers); free(bt->L);
	free(bt);
}

mg_batch* mg_batch_create(int n, void* const targets[], const struct matchgate* const vlists[], const int nlayers[],
	const int* const* const perms[], const int nqubits[], int tune)
{
	if (n < 1 || !targets || !vlists || !nlayers || !perms || !nqubits) { mg_set_error("mg_batch_create: bad arguments"); return NULL; }
	mg_batch* bt = calloc(1, sizeof(*bt));
	if (!bt) return NULL;
	bt->n = n;
	bt->nlayers = malloc(sizeof(int) * n); bt->L = malloc(sizeof(int) * n);
	bt->s = calloc(n, sizeof(seq_circuit)); bt->vlist = calloc(n, sizeof(struct matchgate*));
	mgcu_batch_inst* d = calloc(n, sizeof(mgcu_batch_inst));
	if (!bt->nlayers || !bt->L || !bt->s || !bt->vlist || !d) { free(d); mg_batch_free(bt); return NULL; }
	for (int i = 0; i < n; i++)
	{
		mg_target_handle* th = (mg_target_handle*)targets[i];
		if (!th || th->magic != MG_TARGET_MAGIC || th->L != nqubits[i])
		{
			mg_set_error("mg_batch_create: instance %d needs a GPU target (mg_target_*) on its qubits", i);
			free(d); mg_batch_free(bt); return NULL;
		}
		if (brickwall_seq(vlists[i], nlayers[i], nqubits[i], (const int**)perms[i], &bt->s[i])) { free(d); mg_batch_free(bt); return NULL; }
		bt->nlayers[i] = nlayers[i]; bt->L[i] = nqubits[i];
		bt->vlist[i] = malloc(sizeof(struct matchgate) * nlayers[i]);
		if (!bt->vlist[i]) { free(d); mg_batch_free(bt); return NULL; }
		memcpy(bt->vlist[i], vlists[i], sizeof(struct matchgate) * nlayers[i]);
		d[i].target = th->dev; d[i].L = nqubits[i]; d[i].ngates = bt->s[i].ngates; d[i].wires = bt->s[i].wires;
		d[i].nblocks = nlayers[i]; d[i].block = bt->s[i].block; d[i].want_grad = 1;
	}
	mgcu_lock();
	bt->b = mgcu_batch_create(n, d, mgcu_precision(), tune, 1);
	int r = bt->b ? 0 : MG_ERR_DEVICE;
	for (int i = 0; i < n && !r; i++) r = mgcu_batch_set_gates(bt->b, i, (const mgg*)bt->s[i].gates);
	mgcu_unlock();
	free(d);
	if (r) { mg_batch_free(bt); return NULL; }
	return bt;
}

int mg_batch_set_gates(mg_batch* bt, int i, const struct matchgate vlist[])
{
	if (!bt || i < 0 || i >= bt->n) { mg_set_error("mg_batch_set_gates: bad instance %d", i); return MG_ERR_ARG; }
	const int half = bt->L[i] / 2;
	memcpy(bt->vlist[i], vlist, sizeof(struct matchgate) * bt->nlayers[i]);
	for (int l = 0; l < bt->nlayers[i]; l++)
		for (int p = 0; p < half; p++) bt->s[i].gates[l * half + p] = vlist[l];
	mgcu_lock();
	int r = mgcu_batch_set_gates(bt->b, i, (const mgg*)bt->s[i].gates);
	mgcu_unlock();
	return r;
}

int mg_batch_run(mg_batch* bt)
{
	if (!bt) return MG_ERR_ARG;
	mgcu_lock();
	int r = mgcu_batch_run(bt->b);
	mgcu_unlock();
	return r;
}

int mg_batch_results(mg_batch* bt, int i, numeric* fval, struct matchgate dvlist[], double* grad_vec)
{
	if (!bt || i < 0 || i >= bt->n) { mg_set_error("mg_batch_results: bad instance %d", i); return MG_ERR_ARG; }
	mgcu_lock();
	mgc f;
	int r = mgcu_batch_fetch(bt->b, i, &f, (mgg*)dvlist);
	if (!r && grad_vec) r = mgcu_batch_project(bt->b, i, (const mgg*)bt->vlist[i], grad_vec);
	mgcu_unlock();
	if (!r && fval) *fval = f.re + I * f.im;
	return r;
}

int mg_batch_info(mg_batch* bt, int i, int* target_tile_bits, int* target_passes, int* items)
{
	if (!bt) return MG_ERR_ARG;
	mgcu_lock();
	int r = mgcu_batch_info(bt->b, i, target_tile_bits, target_passes, items);
	mgcu_unlock();
	return r;
}

double mg_batch_time_ms(mg_batch* bt, int steps, int flush_l2)
{
	if (!bt) return -1;
	mgcu_lock();
	double r = mgcu_batch_time_ms(bt->b, steps, flush_l2);
	mgcu_unlock();
	return r;
}
