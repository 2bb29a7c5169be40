/*
 * Request server: evaluations of f, gradients, Hessians and single trust-region steps
 * for brickwall fits against GPU targets, submitted from any thread and served by one
 * worker thread that owns the GPU.
 *
 * Continuous batching: each step the worker takes queued requests, shortest estimated
 * work first (a request queued longer than the aging limit goes first), while their
 * workspace estimates fit the HBM budget and their summed work stays within a step
 * quantum (at least one request per step), so small requests are not held behind large
 * ones.  It runs all f / gradient requests of the step together in one batch (one
 * persistent launch over all their columns), then the Hessian and trust-region requests
 * on device-resident evaluation plans (cached per shape), and completes them; requests
 * that arrive meanwhile wait for the next step.  Targets stay
 * resident (they are the caller's GPU target handles).  The reference has no server;
 * the arithmetic of every request is the library's ordinary evaluation, so a result is
 * the same alone and in a mix up to summation order.
 */
#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "matchgate_target.h"
#include "trust_region.h"
#include "mg_gb300.h"
#include "mg_host.h"
#include "../mg_internal.h"

enum { ST_QUEUED = 0, ST_RUNNING = 1, ST_DONE = 2 };

typedef struct
{
	int kind, L, nlayers, status, state, accepted;
	void* target;
	struct matchgate* vlist;     /* [nlayers] input; TRSTEP: replaced by the accepted point */
	int* perms;                  /* [nlayers * L] */
	double radius, rho;
	double f_re, f_im;
	double* grad_vec;            /* [8 nlayers] */
	double* H;                   /* [(8 nlayers)^2] (HESSIAN, TRSTEP) */
	double t_submit, t_start, t_done;
	size_t est;
	double work;                 /* estimated work, in amplitude-gate updates */
	long step;
} req_t;

/* a device-resident plan kept by the plan lane for later requests of the same shape */
typedef struct
{
	void* target;
	int L, nlayers, what;
	int* perms;
	mg_plan* plan;
	size_t bytes;
	long used;
} pcache_t;

#define NPCACHE 6

struct mg_server
{
	pthread_mutex_t mu;
	pthread_cond_t cv_work, cv_done, cv_lane;
	pthread_t worker, lane;
	int stop, started, lane_started;
	int lane_stop;                 /* set once the worker has exited */
	size_t budget, peak;
	int max_batch;
	req_t** reqs;
	long nreq, cap, next_queued;   /* next_queued: lowest id that may still be queued */
	long steps, batched;
	/* the plan lane: a second thread that serves a step's Hessian and trust-region-step
	 * requests on its own stream while the worker's batch of f / gradient requests runs on
	 * the library's stream, so the two overlap on the GPU */
	req_t** lane_reqs;
	int lane_n, lane_pending;
	void* lane_stream;
	pcache_t cache[NPCACHE];
	long cache_clock;
	size_t cache_bytes;
};

static double now_s(void)
{
	struct timespec t;
	clock_gettime(CLOCK_MONOTONIC, &t);
	return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* device bytes a request holds while it runs (upper estimate of the engine's buffers) */
static size_t estimate(const req_t* r)
{
	const size_t ts = mg_get_precision() == MG_PREC_FP32 ? 8 : 16;
	const size_t S = (size_t)1 << (r->L - 1), N = (size_t)1 << r->L, G = (size_t)r->nlayers * (r->L / 2);
	const size_t blocks = 2 * 152, cap16 = (size_t)16 << 30, cap8 = (size_t)8 << 30;
	const size_t cols = N * S * ts;
	if (r->kind == MG_REQ_TARGET || r->kind == MG_REQ_GRADIENT)
		return (cols < cap16 ? cols : cap16) + blocks * (2 + (r->kind == MG_REQ_GRADIENT ? G : 0)) * S * ts;
	const size_t hc = 2 * N * G * S * ts;
	return (hc < cap16 ? hc : cap16) + (cols < cap8 ? cols : cap8) + 4 * blocks * S * ts;
}

/* amplitude-gate updates: target and fitted sweeps per column (backward counted three
 * times), Hessian items pushing states through the later gates */
static double work_of(const req_t* r)
{
	const double S = (double)((size_t)1 << (r->L - 1)), N = (double)((size_t)1 << r->L), G = (double)r->nlayers * (r->L / 2);
	mgcu_lock();
	const double gu = mgcu_target_sweep_gates(((const mg_target_handle*)r->target)->dev);
	mgcu_unlock();
	double w = N * S * (gu + (r->kind == MG_REQ_TARGET ? 1.0 : 3.0) * G);
	if (r->kind >= MG_REQ_HESSIAN) w += N * S * 8.0 * G * G / 2.0 * (r->kind == MG_REQ_TRSTEP ? 1.1 : 1.0);
	return w;
}

/* work one step may take: about a quarter second of the target sweep at L=16 */
#define STEP_QUANTUM 2.0e11
/* a request queued this long (s) is taken first */
#define AGING_S 2.0

static const int** perm_rows(const req_t* r, const int** rows)
{
	for (int l = 0; l < r->nlayers; l++) rows[l] = r->perms + (size_t)l * r->L;
	return rows;
}

/* the lane's plan for r's shape (target, qubits, layers, wiring, what): a cached one, or a
 * new one kept while the cached plans stay within a quarter of the HBM budget (freeing a
 * plan waits for the whole device, so the lane keeps recent ones) */
static mg_plan* lane_plan(mg_server* sv, const req_t* r, int what)
{
	const size_t pb = sizeof(int) * (size_t)r->nlayers * r->L;
	for (int i = 0; i < NPCACHE; i++)
	{
		pcache_t* c = &sv->cache[i];
		if (c->plan && c->target == r->target && c->L == r->L && c->nlayers == r->nlayers && c->what == what && !memcmp(c->perms, r->perms, pb))
		{
			c->used = ++sv->cache_clock;
			return c->plan;
		}
	}
	const int** rows = malloc(sizeof(int*) * r->nlayers);
	if (!rows) return NULL;
	mg_plan* pl = mg_plan_brickwall(mg_target_apply, r->target, r->vlist, r->nlayers, r->L, perm_rows(r, rows), what);
	free(rows);
	if (!pl) return NULL;
	const size_t bytes = r->est;
	/* evict least recently used plans until this one fits the slots and the byte cap */
	for (;;)
	{
		int nused = 0, lru = -1;
		for (int i = 0; i < NPCACHE; i++)
			if (sv->cache[i].plan) { nused++; if (lru < 0 || sv->cache[i].used < sv->cache[lru].used) lru = i; }
		if (nused < NPCACHE && sv->cache_bytes + bytes <= sv->budget / 4) break;
		if (lru < 0) break;
		mg_plan_free(sv->cache[lru].plan);
		free(sv->cache[lru].perms);
		sv->cache_bytes -= sv->cache[lru].bytes;
		memset(&sv->cache[lru], 0, sizeof(pcache_t));
	}
	for (int i = 0; i < NPCACHE; i++)
	{
		pcache_t* c = &sv->cache[i];
		if (c->plan) continue;
		if (sv->cache_bytes + bytes > sv->budget / 4) break;
		c->perms = malloc(pb);
		if (!c->perms) break;
		memcpy(c->perms, r->perms, pb);
		c->target = r->target; c->L = r->L; c->nlayers = r->nlayers; c->what = what; c->plan = pl; c->bytes = bytes;
		c->used = ++sv->cache_clock;
		sv->cache_bytes += bytes;
		return pl;
	}
	return pl;   /* not cached: the caller frees it */
}

static int lane_cached(const mg_server* sv, const mg_plan* pl)
{
	for (int i = 0; i < NPCACHE; i++) if (sv->cache[i].plan == pl) return 1;
	return 0;
}

/* f, projected gradient and Hessian (what = MG_EVAL_*) of r's current gates on a lane plan;
 * the wait for the GPU happens outside the library lock, so the worker's batch can be
 * issued and collected meanwhile */
static int eval_plan(mg_server* sv, req_t* r, int what, double* f, double* grad_vec, double* H)
{
	mg_plan* pl = lane_plan(sv, r, what);
	if (!pl) return MG_ERR_DEVICE;
	int rc = mg_plan_set_gates(pl, r->vlist);
	if (!rc) rc = mg_plan_run(pl);
	if (!rc) rc = mgcu_stream_sync();
	numeric fc = 0;
	if (!rc) rc = mg_plan_results(pl, &fc, NULL, NULL, grad_vec, H);
	if (!lane_cached(sv, pl)) mg_plan_free(pl);
	if (!rc) { f[0] = creal(fc); f[1] = cimag(fc); }
	return rc;
}

/* one Riemannian trust-region step (the loop body of src/trust_region.c:258-305) */
static int tr_step(mg_server* sv, req_t* r)
{
	const int n = 8 * r->nlayers;
	double f0[2], f1[2];
	double* eta = malloc(sizeof(double) * n);
	double* heta = malloc(sizeof(double) * n);
	struct matchgate* vnew = malloc(sizeof(struct matchgate) * r->nlayers);
	struct matchgate* vold = r->vlist;
	int rc = (!eta || !heta || !vnew) ? MG_ERR_ALLOC : 0;
	if (!rc) rc = eval_plan(sv, r, MG_EVAL_HESSIAN, f0, r->grad_vec, r->H);
	if (!rc)
	{
		struct rtr_params rp;
		set_rtr_default_params(n, &rp);
		struct truncated_cg_params p = rp.tcg_params;
		const bool on_boundary = truncated_cg_hmat(r->grad_vec, r->H, n, r->radius, &p, eta);
		for (int l = 0; l < r->nlayers; l++) retract_matchgate(&vold[l], eta + 8 * l, &vnew[l]);
		double gd = 0, eh = 0;
		for (int i = 0; i < n; i++)
		{
			double s = 0;
			for (int j = 0; j < n; j++) s += r->H[(size_t)i * n + j] * eta[j];
			heta[i] = s;
			gd += r->grad_vec[i] * eta[i];
			eh += eta[i] * s;
		}
		r->vlist = vnew;
		rc = eval_plan(sv, r, MG_EVAL_TARGET, f1, NULL, NULL);
		r->vlist = vold;
		if (!rc)
		{
			/* the target function is Re f (src/mg_brickwall_opt.c:20-31) */
			const double rho = (f1[0] - f0[0]) / (gd + 0.5 * eh);
			r->rho = rho;
			if (rho < 0.25) r->radius *= 0.25;
			else if (rho > 0.75 && on_boundary) r->radius = fmin(2 * r->radius, rp.maxradius);
			r->accepted = rho > rp.rho_trust;
			if (r->accepted) { memcpy(r->vlist, vnew, sizeof(struct matchgate) * r->nlayers); r->f_re = f1[0]; r->f_im = f1[1]; }
			else { r->f_re = f0[0]; r->f_im = f0[1]; }
		}
	}
	free(eta); free(heta); free(vnew);
	return rc;
}

/* the f / gradient requests of one step, as one batch on the library's stream: issued under
 * the library lock, waited for outside it (the plan lane keeps issuing meanwhile), then
 * collected.  Returns the batch, freed by the caller once the lane is idle (freeing device
 * memory waits for the whole GPU). */
static mgcu_batch* run_batch(req_t** rs, int n)
{
	mgcu_batch_inst* d = calloc(n, sizeof(mgcu_batch_inst));
	seq_circuit* s = calloc(n, sizeof(seq_circuit));
	int rc = (!d || !s) ? MG_ERR_ALLOC : 0;
	int built = 0;
	for (int i = 0; i < n && !rc; i++, built++)
	{
		const int** rows = malloc(sizeof(int*) * rs[i]->nlayers);
		if (!rows) { rc = MG_ERR_ALLOC; break; }
		rc = brickwall_seq(rs[i]->vlist, rs[i]->nlayers, rs[i]->L, perm_rows(rs[i], rows), &s[i]);
		free(rows);
		if (rc) break;
		d[i].target = ((mg_target_handle*)rs[i]->target)->dev; d[i].L = rs[i]->L; d[i].ngates = s[i].ngates;
		d[i].wires = s[i].wires; d[i].nblocks = rs[i]->nlayers; d[i].block = s[i].block;
		d[i].want_grad = rs[i]->kind == MG_REQ_GRADIENT;
	}
	mgcu_batch* b = NULL;
	if (!rc)
	{
		mgcu_lock();
		/* a step's batch runs once: no tile timing, no graph */
		b = mgcu_batch_create(n, d, mgcu_precision(), 0, 0);
		rc = b ? 0 : MG_ERR_DEVICE;
		for (int i = 0; i < n && !rc; i++) rc = mgcu_batch_set_gates(b, i, (const mgg*)s[i].gates);
		if (!rc) rc = mgcu_batch_issue(b);
		mgcu_unlock();
		if (!rc) rc = mgcu_stream_sync();
		mgcu_lock();
		for (int i = 0; i < n && !rc; i++)
		{
			mgc f;
			rc = mgcu_batch_fetch(b, i, &f, NULL);
			if (!rc) { rs[i]->f_re = f.re; rs[i]->f_im = f.im; }
			if (!rc && rs[i]->kind == MG_REQ_GRADIENT) rc = mgcu_batch_project(b, i, (const mgg*)rs[i]->vlist, rs[i]->grad_vec);
		}
		mgcu_unlock();
	}
	for (int i = 0; i < built; i++) seq_free(&s[i]);
	for (int i = 0; i < n; i++) rs[i]->status = rc;
	free(d); free(s);
	return b;
}

/* mark r done (its results are in place) and wake the waiters */
static void complete(mg_server* sv, req_t* r)
{
	pthread_mutex_lock(&sv->mu);
	r->t_done = now_s();
	r->state = ST_DONE;
	pthread_cond_broadcast(&sv->cv_done);
	pthread_mutex_unlock(&sv->mu);
}

/* the plan lane: serves the Hessian and trust-region-step requests each step hands it */
static void* lane_worker(void* arg)
{
	mg_server* sv = (mg_server*)arg;
	mgcu_stream_set(sv->lane_stream);
	for (;;)
	{
		pthread_mutex_lock(&sv->mu);
		while (!sv->lane_pending && !sv->lane_stop) pthread_cond_wait(&sv->cv_lane, &sv->mu);
		if (!sv->lane_pending) { pthread_mutex_unlock(&sv->mu); break; }
		req_t** rs = sv->lane_reqs;
		const int n = sv->lane_n;
		pthread_mutex_unlock(&sv->mu);
		for (int i = 0; i < n; i++)
		{
			req_t* r = rs[i];
			if (r->kind == MG_REQ_HESSIAN)
			{
				double f[2] = { 0, 0 };
				r->status = eval_plan(sv, r, MG_EVAL_HESSIAN, f, r->grad_vec, r->H);
				r->f_re = f[0]; r->f_im = f[1];
			}
			else r->status = tr_step(sv, r);
			complete(sv, r);
		}
		pthread_mutex_lock(&sv->mu);
		sv->lane_pending = 0;
		pthread_cond_broadcast(&sv->cv_lane);
		pthread_mutex_unlock(&sv->mu);
	}
	for (int i = 0; i < NPCACHE; i++)
		if (sv->cache[i].plan) { mg_plan_free(sv->cache[i].plan); free(sv->cache[i].perms); }
	memset(sv->cache, 0, sizeof(sv->cache));
	mgcu_stream_set(NULL);
	return NULL;
}

static void* worker(void* arg)
{
	mg_server* sv = (mg_server*)arg;
	req_t** step = malloc(sizeof(req_t*) * (size_t)sv->max_batch);
	req_t** bat = malloc(sizeof(req_t*) * (size_t)sv->max_batch);
	req_t** heavy = malloc(sizeof(req_t*) * (size_t)sv->max_batch);
	for (;;)
	{
		pthread_mutex_lock(&sv->mu);
		int n = 0;
		for (;;)
		{
			size_t used = 0;
			double work = 0;
			n = 0;
			const double tnow = now_s();
			for (;;)
			{
				/* next: the oldest request past the aging limit, else the least work */
				req_t* best = NULL;
				for (long id = sv->next_queued; id < sv->nreq; id++)
				{
					req_t* r = sv->reqs[id];
					if (r->state != ST_QUEUED) continue;
					if (r->est > sv->budget)
					{
						/* can never fit: fail it */
						r->status = MG_ERR_ARG; r->state = ST_DONE; r->t_start = r->t_done = now_s();
						continue;
					}
					if (r->work < 0) r->work = work_of(r);
					if (used + r->est > sv->budget || (n > 0 && work + r->work > STEP_QUANTUM)) continue;
					const int aged = tnow - r->t_submit > AGING_S, best_aged = best && tnow - best->t_submit > AGING_S;
					if (!best || (aged && !best_aged) || (aged == best_aged && !aged && r->work < best->work)) best = r;
				}
				if (!best || n >= sv->max_batch) break;
				best->state = ST_RUNNING;
				used += best->est;
				work += best->work;
				step[n++] = best;
			}
			while (sv->next_queued < sv->nreq && sv->reqs[sv->next_queued]->state != ST_QUEUED) sv->next_queued++;
			if (n > 0 || sv->stop) { if (used > sv->peak) sv->peak = used; break; }
			pthread_cond_broadcast(&sv->cv_done);
			pthread_cond_wait(&sv->cv_work, &sv->mu);
		}
		if (n == 0 && sv->stop) { pthread_cond_broadcast(&sv->cv_done); pthread_mutex_unlock(&sv->mu); break; }
		const double t0 = now_s();
		const long stepno = sv->steps++;
		for (int i = 0; i < n; i++) { step[i]->state = ST_RUNNING; step[i]->t_start = t0; step[i]->step = stepno; }
		pthread_mutex_unlock(&sv->mu);

		int nb = 0, nh = 0;
		for (int i = 0; i < n; i++)
			if (step[i]->kind == MG_REQ_TARGET || step[i]->kind == MG_REQ_GRADIENT) bat[nb++] = step[i];
			else heavy[nh++] = step[i];
		if (nh > 0)
		{
			/* the Hessian and trust-region-step requests go to the plan lane, which runs them
			 * on its own stream while this thread's batch runs */
			pthread_mutex_lock(&sv->mu);
			sv->lane_reqs = heavy; sv->lane_n = nh; sv->lane_pending = 1;
			pthread_cond_broadcast(&sv->cv_lane);
			pthread_mutex_unlock(&sv->mu);
		}
		mgcu_batch* b = nb > 0 ? run_batch(bat, nb) : NULL;
		for (int i = 0; i < nb; i++) complete(sv, bat[i]);
		pthread_mutex_lock(&sv->mu);
		while (sv->lane_pending) pthread_cond_wait(&sv->cv_lane, &sv->mu);
		sv->batched += nb;
		pthread_mutex_unlock(&sv->mu);
		if (b) { mgcu_lock(); mgcu_batch_destroy(b); mgcu_unlock(); }
	}
	free(step); free(bat); free(heavy);
	return NULL;
}

mg_server* mg_server_create(size_t hbm_budget_bytes, int max_batch)
{
	mg_server* sv = calloc(1, sizeof(*sv));
	if (!sv) return NULL;
	sv->budget = hbm_budget_bytes;
	sv->max_batch = max_batch > 0 ? max_batch : 256;
	pthread_mutex_init(&sv->mu, NULL);
	pthread_cond_init(&sv->cv_work, NULL);
	pthread_cond_init(&sv->cv_done, NULL);
	pthread_cond_init(&sv->cv_lane, NULL);
	sv->lane_stream = mgcu_stream_create();
	if (!sv->lane_stream || pthread_create(&sv->lane, NULL, lane_worker, sv) != 0)
	{
		if (sv->lane_stream) mgcu_stream_destroy(sv->lane_stream);
		mg_set_error("mg_server_create: could not start the plan lane (%s)", mg_last_error());
		free(sv);
		return NULL;
	}
	sv->lane_started = 1;
	if (pthread_create(&sv->worker, NULL, worker, sv) != 0)
	{
		pthread_mutex_lock(&sv->mu);
		sv->lane_stop = 1;
		pthread_cond_broadcast(&sv->cv_lane);
		pthread_mutex_unlock(&sv->mu);
		pthread_join(sv->lane, NULL);
		mgcu_stream_destroy(sv->lane_stream);
		mg_set_error("mg_server_create: could not start the worker thread");
		free(sv);
		return NULL;
	}
	sv->started = 1;
	return sv;
}

long mg_server_submit(mg_server* sv, const mg_request* q)
{
	if (!sv || !q || !q->target || !q->vlist || !q->perms || q->nlayers < 1 || q->nqubits < 4 || q->nqubits % 2
		|| q->kind < MG_REQ_TARGET || q->kind > MG_REQ_TRSTEP)
	{
		mg_set_error("mg_server_submit: bad request");
		return MG_ERR_ARG;
	}
	const mg_target_handle* th = (const mg_target_handle*)q->target;
	if (th->magic != MG_TARGET_MAGIC || th->L != q->nqubits)
	{
		mg_set_error("mg_server_submit: the target must be a GPU target (mg_target_*) on the request's qubits");
		return MG_ERR_ARG;
	}
	req_t* r = calloc(1, sizeof(req_t));
	if (!r) return MG_ERR_ALLOC;
	const int n = 8 * q->nlayers;
	r->kind = q->kind; r->L = q->nqubits; r->nlayers = q->nlayers; r->target = q->target; r->radius = q->radius;
	r->vlist = malloc(sizeof(struct matchgate) * q->nlayers);
	r->perms = malloc(sizeof(int) * (size_t)q->nlayers * q->nqubits);
	r->grad_vec = calloc(n, sizeof(double));
	if (q->kind >= MG_REQ_HESSIAN) r->H = calloc((size_t)n * n, sizeof(double));
	if (!r->vlist || !r->perms || !r->grad_vec || (q->kind >= MG_REQ_HESSIAN && !r->H))
	{
		free(r->vlist); free(r->perms); free(r->grad_vec); free(r->H); free(r);
		return MG_ERR_ALLOC;
	}
	memcpy(r->vlist, q->vlist, sizeof(struct matchgate) * q->nlayers);
	memcpy(r->perms, q->perms, sizeof(int) * (size_t)q->nlayers * q->nqubits);
	r->est = estimate(r);
	r->work = -1;   /* computed by the worker (it may need the library lock) */
	pthread_mutex_lock(&sv->mu);
	if (sv->nreq == sv->cap)
	{
		const long nc = sv->cap ? 2 * sv->cap : 256;
		req_t** nr = realloc(sv->reqs, sizeof(req_t*) * (size_t)nc);
		if (!nr) { pthread_mutex_unlock(&sv->mu); free(r->vlist); free(r->perms); free(r->grad_vec); free(r->H); free(r); return MG_ERR_ALLOC; }
		sv->reqs = nr; sv->cap = nc;
	}
	const long id = sv->nreq++;
	r->t_submit = now_s();
	r->state = ST_QUEUED;
	sv->reqs[id] = r;
	pthread_cond_signal(&sv->cv_work);
	pthread_mutex_unlock(&sv->mu);
	return id;
}

int mg_server_wait(mg_server* sv, long id)
{
	if (!sv || id < 0) return MG_ERR_ARG;
	pthread_mutex_lock(&sv->mu);
	if (id >= sv->nreq) { pthread_mutex_unlock(&sv->mu); mg_set_error("mg_server_wait: unknown request %ld", id); return MG_ERR_ARG; }
	while (sv->reqs[id]->state != ST_DONE) pthread_cond_wait(&sv->cv_done, &sv->mu);
	const int st = sv->reqs[id]->status;
	pthread_mutex_unlock(&sv->mu);
	return st;
}

int mg_server_done(mg_server* sv, long id)
{
	if (!sv || id < 0) return MG_ERR_ARG;
	pthread_mutex_lock(&sv->mu);
	const int d = id < sv->nreq && sv->reqs[id]->state == ST_DONE;
	pthread_mutex_unlock(&sv->mu);
	return d;
}

int mg_server_result(mg_server* sv, long id, numeric* fval, double* grad_vec, double* H, struct matchgate vlist[],
	double* radius, int* accepted, double times[3], long* step)
{
	const int st = mg_server_wait(sv, id);
	pthread_mutex_lock(&sv->mu);
	const req_t* r = sv->reqs[id];
	const int n = 8 * r->nlayers;
	if (fval) *fval = r->f_re + I * r->f_im;
	if (grad_vec) memcpy(grad_vec, r->grad_vec, sizeof(double) * n);
	if (H && r->H) memcpy(H, r->H, sizeof(double) * (size_t)n * n);
	if (vlist) memcpy(vlist, r->vlist, sizeof(struct matchgate) * r->nlayers);
	if (radius) *radius = r->radius;
	if (accepted) *accepted = r->accepted;
	if (times) { times[0] = r->t_submit; times[1] = r->t_start; times[2] = r->t_done; }
	if (step) *step = r->step;
	pthread_mutex_unlock(&sv->mu);
	return st;
}

void mg_server_stats(mg_server* sv, long* steps, long* batched, size_t* peak_bytes)
{
	pthread_mutex_lock(&sv->mu);
	if (steps) *steps = sv->steps;
	if (batched) *batched = sv->batched;
	if (peak_bytes) *peak_bytes = sv->peak;
	pthread_mutex_unlock(&sv->mu);
}

void mg_server_free(mg_server* sv)
{
	if (!sv) return;
	if (sv->started)
	{
		pthread_mutex_lock(&sv->mu);
		sv->stop = 1;
		pthread_cond_signal(&sv->cv_work);
		pthread_mutex_unlock(&sv->mu);
		pthread_join(sv->worker, NULL);
	}
	if (sv->lane_started)
	{
		/* after the worker: it may still hand the lane the requests it drains */
		pthread_mutex_lock(&sv->mu);
		sv->lane_stop = 1;
		pthread_cond_broadcast(&sv->cv_lane);
		pthread_mutex_unlock(&sv->mu);
		pthread_join(sv->lane, NULL);
		mgcu_stream_destroy(sv->lane_stream);
	}
	for (long i = 0; i < sv->nreq; i++)
	{
		req_t* r = sv->reqs[i];
		free(r->vlist); free(r->perms); free(r->grad_vec); free(r->H); free(r);
	}
	free(sv->reqs);
	pthread_cond_destroy(&sv->cv_work);
	pthread_cond_destroy(&sv->cv_done);
	pthread_cond_destroy(&sv->cv_lane);
	pthread_mutex_destroy(&sv->mu);
	free(sv);
}
