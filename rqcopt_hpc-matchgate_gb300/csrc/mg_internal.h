/*
 * Internal interface between the host C layer (csrc/host, which implements the
 * reference-compatible API) and the CUDA layer (csrc/cuda).  Plain C types only.
 *
 * Every mgcu_* function returns 0 on success and MG_ERR_DEVICE (-5) on a CUDA error
 * (the message is kept for mg_last_error() and printed to stderr), or -1 when a
 * device allocation fails.
 */
#pragma once

#include <stddef.h>
#include "mg_algebra.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MG_ERR_ALLOC  (-1)
#define MG_ERR_UFUNC  (-2)
#define MG_ERR_DEVICE (-5)
#define MG_ERR_ARG    (-6)

/* precision identifiers (same values as MG_PREC_* of mg_gb300.h) */
#define MG_PREC_FP64_ID  0
#define MG_PREC_MIXED_ID 1
#define MG_PREC_FP32_ID  2

/* option identifiers (same values as MG_OPT_* of mg_gb300.h) */
#define MG_OPT_TILE_BITS_ID     1
#define MG_OPT_THREADS_ID       2
#define MG_OPT_CHUNK_COLUMNS_ID 3
#define MG_OPT_CTAS_PER_SM_ID   4
#define MG_OPT_TARGET_TILE_BITS_ID 5
#define MG_OPT_TARGET_THREADS_ID   6
#define MG_OPT_TARGET_COLUMNS_ID   7
#define MG_OPT_TRANSLATIONAL_INVARIANCE_ID 8
#define MG_OPT_TARGET_DENSE_ID  9
#define MG_OPT_HOST_THREADS_ID  10
#define MG_OPT_FIT_CACHE_ID     11
#define MG_OPT_TARGET_TUNE_ID   12
#define MG_OPT_HESS_GROUP_ID    13
#define MG_OPT_FIT_RESIDENT_ID  14
#define MG_NOPTIONS             14

/* ---- runtime ---- */
/* streams: each host thread issues its GPU work on its own stream when it selected one
 * (mgcu_stream_set; NULL: the library's stream); mgcu_stream_sync waits for the calling
 * thread's stream and needs no library lock */
void* mgcu_stream_create(void);
void mgcu_stream_set(void* stream);
int mgcu_stream_sync(void);
void mgcu_stream_destroy(void* stream);
void mg_set_error(const char* fmt, ...);
const char* mg_last_error(void);
void mgcu_lock(void);
void mgcu_unlock(void);
int mgcu_precision(void);
long mgcu_option(int option);

/* ---- per-vector primitives on host buffers (FP64, full 2^L vectors) ---- */
/* out = G psi for nstates interleaved vectors (nstates = 1: a plain vector) */
int mgcu_prim_apply(const mgg* g, int i, int j, int L, int nstates, const mgc* psi, mgc* out);
int mgcu_prim_backward(const mgg* g, int i, int j, int L, const mgc* psi, const mgc* dpsi_out, mgc* dpsi, mgg* dg);
int mgcu_prim_backward_array(const mgg* g, int i, int j, int L, int nstates, const mgc* psi, const mgc* dpsi_out, mgg* dgs);
/* nout = 8 (matchgate entries) or 16 (general 4x4 gate entries) */
int mgcu_prim_placeholder(int i, int j, int L, int nout, const mgc* psi, mgc* out);
/* sequential circuits on one vector: cache (host, ngates x 2^L) may be NULL for apply */
int mgcu_circuit_forward(const mgg* gates, const int* wires, int ngates, int L, const mgc* psi, mgc* cache, mgc* out);
int mgcu_circuit_backward(const mgg* gates, const int* wires, int ngates, int L, const mgc* cache, const mgc* dpsi_out,
	mgc* dpsi, mgg* dgates);
/* Hessian of one column for a brickwall (per-layer blocks, optional translation
 * invariance): reference src/matchgate_brickwall.c:137-260 / :308-435 */
int mgcu_brickwall_backward_hessian(const mgg* vlist, int nlayers, const int* perms, int L, int ti, const mgc* cache,
	const mgc* dpsi_out, mgc* dpsi, mgg* dvlist, mgc* hess);

/* ---- GPU target maps ---- */
typedef struct mgcu_target mgcu_target;
mgcu_target* mgcu_target_circuit(const mgg* gates, const int* wires, int ngates, int L);
mgcu_target* mgcu_target_dense(const mgc* U, int L);
void mgcu_target_destroy(mgcu_target* t);
int mgcu_target_apply(mgcu_target* t, const mgc* psi, mgc* out);      /* host vectors */
int mgcu_target_L(const mgcu_target* t);
void mgcu_target_set_resident(mgcu_target* t, int enable);
int mgcu_target_resident(const mgcu_target* t);
double mgcu_device_free_bytes(void);
/* host layer: residency of a GPU target handle (-1: not a GPU circuit target) */
int mgh_target_resident(void* udata);
int mgcu_target_sweep_gates(mgcu_target* t);
int mgcu_target_conserves_weight(mgcu_target* t);

/* ---- batched evaluation plans (the hot path) ---- */
typedef struct
{
	int L;
	int ngates;            /* fitted circuit W in sequential order */
	const int* wires;      /* [2*ngates] */
	int nblocks;           /* gradient/Hessian blocks; gate g belongs to block[g] */
	const int* block;      /* [ngates]; NULL means block[g] = g */
	int want_grad;
	int want_hess;
	int nplace;            /* Hessian placements (gate indices) and their weights */
	const int* place;      /* [nplace] */
	const double* place_w; /* [nplace][ngates]: weight of (placement p, later gate l) */
	mgcu_target* target;   /* GPU target; NULL: columns are supplied per chunk from the host */
	int precision;
} mgcu_plan_desc;

typedef struct mgcu_plan mgcu_plan;
mgcu_plan* mgcu_plan_create(const mgcu_plan_desc* d);
void mgcu_plan_destroy(mgcu_plan* p);
int mgcu_plan_set_gates(mgcu_plan* p, const mgg* gates);      /* [ngates] host gates */
int mgcu_plan_begin(mgcu_plan* p);                              /* zero accumulators */
/* accumulate columns b in [b0, b1); host_cols (or NULL for a GPU target) holds
 * -conj(U e_b) restricted to the parity sector of b, [b1-b0][2^(L-1)] */
int mgcu_plan_columns(mgcu_plan* p, long b0, long b1, const mgc* host_cols);
/* final reductions on the GPU; outputs stay on the device */
int mgcu_plan_finish(mgcu_plan* p);
/* copy results: f, per-block gradients [nblocks], complex Hessian [(8 nblocks)^2] */
int mgcu_plan_fetch(mgcu_plan* p, mgc* f, mgg* dblocks, mgc* hess);
/* project on the GPU (layer blocks): grad_vec [8 nblocks] and H [(8 nblocks)^2] */
int mgcu_plan_project(mgcu_plan* p, const mgg* vblocks, double* grad_vec, double* H);
long mgcu_plan_chunk_columns(const mgcu_plan* p);
double mgcu_plan_time_ms(mgcu_plan* p, long b0, long b1, int steps, int flush_l2);

/* ---- batches of instances (f and block gradients), persistent launches + CUDA graph ---- */
typedef struct
{
	mgcu_target* target;   /* GPU circuit target on L qubits */
	int L;
	int ngates;            /* fitted circuit in sequential order */
	const int* wires;      /* [2*ngates] */
	int nblocks;
	const int* block;      /* [ngates] */
	int want_grad;         /* 0: f only */
} mgcu_batch_inst;
typedef struct mgcu_batch mgcu_batch;
mgcu_batch* mgcu_batch_create(int n, const mgcu_batch_inst* insts, int precision, int tune, int use_graph);
void mgcu_batch_destroy(mgcu_batch* b);
int mgcu_batch_set_gates(mgcu_batch* b, int i, const mgg* gates);   /* [ngates_i] */
int mgcu_batch_run(mgcu_batch* b);
int mgcu_batch_issue(mgcu_batch* b);     /* queued on the calling thread's stream, no wait */
int mgcu_batch_fetch(mgcu_batch* b, int i, mgc* f, mgg* dblocks);
int mgcu_batch_project(mgcu_batch* b, int i, const mgg* vblocks, double* grad_vec);
int mgcu_batch_info(const mgcu_batch* b, int i, int* target_tile_bits, int* target_passes, int* items);
double mgcu_batch_time_ms(mgcu_batch* b, int steps, int flush_l2);
int mgcu_plan_target_kernel_ms(mgcu_plan* p, double* ms, long* launches);
void mgcu_plan_target_config(const mgcu_plan* p, int* cfg);

/* ---- FP64 algebra on the GPU ---- */
int mgcu_retract(const mgg* u, const double* eta, int n, mgg* v);
/* truncated CG (src/trust_region.c:88-146); returns 1 on the boundary, 0 inside, < 0 on error */
int mgcu_truncated_cg(const double* grad, const double* hess, int n, double radius, int maxiter, double abstol, double reltol, double* z);
/* y = H x for a dense n x n row-major matrix */
int mgcu_matvec(const double* H, const double* x, int n, double* y);
/* out = U psi for a dense 2^L x 2^L complex matrix U already on the GPU */
int mgcu_dense_matvec(const void* U_dev, int L, const mgc* psi, mgc* out);

/* ---- instrumentation ---- */
long mgcu_launch_count(void);
double mgcu_fp32_peak_gflops(void);
double mgcu_fp64_peak_gflops(void);

#ifdef __cplusplus
}
#endif
