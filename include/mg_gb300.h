/*
 * Extensions of the GB300 matchgate library beyond the reference's C API.
 * Nothing here changes the meaning of a reference entry point; these add
 * precision control, GPU-resident target maps, device-resident evaluation plans
 * for callers that keep their data on the GPU, and results the reference only
 * computes inside larger calls.
 */
#pragma once

#include "matchgate_target.h"
#include "trust_region.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------------
 * Precision of the batched evaluations (matchgate_target.h entry points).
 *   MG_PREC_FP64  complex128 sweeps and sums (default; matches the reference)
 *   MG_PREC_MIXED float-float sweeps (pairs of FP32, about 48 significant bits),
 *                 compensated FP32 products and sums, FP64 final reductions
 *   MG_PREC_FP32  complex FP32 sweeps, compensated FP32 sums into FP64
 * Projection, retraction and the trust-region subproblem always run in FP64.
 * --------------------------------------------------------------------------------- */
enum { MG_PREC_FP64 = 0, MG_PREC_MIXED = 1, MG_PREC_FP32 = 2 };
int mg_set_precision(int precision);
int mg_get_precision(void);

/* Tuning options (0 = automatic).  TILE_BITS: log2 of amplitudes per shared-memory
 * tile; THREADS: threads per block; CHUNK_COLUMNS: basis columns per batch when
 * columns are materialised from a host map or a Hessian is requested;
 * CTAS_PER_SM: resident blocks per SM for the persistent grid; TARGET_TILE_BITS and
 * TARGET_THREADS: the same two for the sweep of a GPU circuit target (default: TILE_BITS
 * and its block size; at most 2^13 amplitudes of 16 B and 512 threads); TARGET_COLUMNS: 2 sweeps
 * two basis columns of equal parity per block (256 threads), sharing the per-gate work.
 * TRANSLATIONAL_INVARIANCE: 1 makes matchgate_brickwall_unitary_target_gradient_hessian, its
 * parallel_ twin, matchgate_brickwall_unitary_target_gradient_vector_hessian_matrix and
 * mg_optimize_brickwall use the translation-invariant Hessian -- what building the reference
 * with -DTRANSLATIONAL_INVARIANCE does to the same entry points (src/matchgate_target.c:478,
 * 715, 819); 0 (default) is the reference's plain build.
 * TARGET_DENSE: 1 sweeps every amplitude of a GPU circuit target even when all its gates
 * conserve the Hamming weight (by default such targets are swept on the amplitudes of the
 * basis column's weight only; both give bit-identical results).
 * HOST_THREADS: host threads that call a caller's linear_func (a host map, not a GPU target)
 * concurrently, one basis column per call, as the reference's OpenMP threads do; the map must
 * be re-entrant (it is for the reference's own maps).  0 = the online cores; results do not
 * depend on the count.
 * FIT_CACHE: how a gradient evaluation gets each fitted gate's input in the backward sweep.
 * 0 or 1 (default): the reference's cache of every gate's input state
 * (src/matchgate_brickwall.c:52-127); 2: only each pass's output state is kept and the inputs
 * are recovered with the gates' block inverses (one state per pass and block instead of one
 * per gate, much less device memory and traffic, but a third more arithmetic and about 25 %
 * slower in float-float at L=16-18; gates that are not invertible fall back to the cache).
 * Hessian evaluations always cache.
 * TARGET_TUNE: how the block size of a GPU circuit target's sweep is chosen when
 * TARGET_THREADS is 0.  0 (default): by timing the candidates (128 or 256 threads, and for
 * the full sweep 512) on one resident wave of columns when the trace has at least 2^14
 * columns, once per target, precision and tile size; 1: never (128 threads); 2: always.
 * The candidates give bit-identical results.
 * HESS_GROUP: how a plain Hessian of parameter blocks shared by several gates (the per-layer
 * brickwall Hessian) is computed.  0 (default): one forward-mode sweep per basis column,
 * block and entry, which adds each of the block's gates' placeholder terms as it passes them
 * (a sixth of the gate steps at L=16 with 5 layers); 1: one sweep per gate and entry, the
 * reference's placements (src/matchgate_brickwall.c:177-231).  The two agree to rounding.
 * FIT_RESIDENT: 0 (default) lets mg_optimize_brickwall / mg_optimize_circuit keep a GPU
 * circuit target's columns on the GPU for the duration of the fit (the target is fixed
 * there) when they take at most a quarter of the free device memory (2^(2L-1) x 16 bytes:
 * 32 GiB at L=16), so only the first evaluation sweeps the target; 1 sweeps it in every
 * evaluation, as the reference applies its target map each time.  Results are the same. */
enum { MG_OPT_TILE_BITS = 1, MG_OPT_THREADS = 2, MG_OPT_CHUNK_COLUMNS = 3, MG_OPT_CTAS_PER_SM = 4,
       MG_OPT_TARGET_TILE_BITS = 5, MG_OPT_TARGET_THREADS = 6, MG_OPT_TARGET_COLUMNS = 7,
       MG_OPT_TRANSLATIONAL_INVARIANCE = 8, MG_OPT_TARGET_DENSE = 9, MG_OPT_HOST_THREADS = 10,
       MG_OPT_FIT_CACHE = 11, MG_OPT_TARGET_TUNE = 12, MG_OPT_HESS_GROUP = 13, MG_OPT_FIT_RESIDENT = 14 };
int mg_set_option(int option, long value);
long mg_get_option(int option);

/* Last error message of this thread's most recent failing call ("" if none). */
const char* mg_last_error(void);

/* ---------------------------------------------------------------------------------
 * GPU-resident target maps.  Each constructor returns the `udata` to pass together
 * with `mg_target_apply` as the (ufunc, udata) pair of any matchgate_target.h call;
 * the library recognises the pair and applies U on the GPU per basis column instead
 * of calling a host function 2^L times.  mg_target_apply itself applies U to a host
 * vector (on the GPU), so the pair also works wherever a linear_func is called.
 * --------------------------------------------------------------------------------- */
int mg_target_apply(const struct statevector* restrict psi, void* udata, struct statevector* restrict psi_out);
void* mg_target_brickwall(const struct matchgate ulist[], int ulayers, const int* uperms[], int nqubits);
void* mg_target_circuit(const struct matchgate gates[], int ngates, const int wires[], int nqubits);
void* mg_target_dense(const numeric* U, int nqubits);   /* row-major 2^L x 2^L */
void mg_target_free(void* udata);
/* Keep the conjugated target columns -conj(U e_b) resident in GPU memory after their
 * first use (about 2^(2L-1) amplitudes), so later evaluations against the same target
 * skip re-applying U.  Off by default. */
int mg_target_set_resident(void* udata, int enable);
/* Number of gates the GPU sweep of a circuit target applies per column: the circuit's
 * gates less the fermionic swaps removed by relabelling wires (paired swaps that
 * restore the qubit order; the other gates then carry Jordan-Wigner strings), plus
 * any controlled-Z left over.  -1 for a dense target or an invalid handle. */
int mg_target_sweep_gates(void* udata);
/* 1 when every gate of a circuit target conserves the Hamming weight (no corner block mixes
 * |00> and |11>: hopping and interaction terms of particle-conserving Hamiltonians, fermionic
 * swaps).  U e_b then has nonzero amplitudes only at indices of the weight of b, and the GPU
 * sweep visits only those (unless MG_OPT_TARGET_DENSE is set): C(2L, L) amplitude-columns per
 * trace instead of 2^(2L-1), with bit-identical results.  0 otherwise (also for dense
 * targets), -1 for an invalid handle. */
int mg_target_conserves_weight(void* udata);

/* ---------------------------------------------------------------------------------
 * Native trust-region fit (the loop of riemannian_trust_region_optimize_hmat,
 * src/trust_region.c:235-306, driven as optimize_matchgate_brickwall_circuit_hmat,
 * src/mg_brickwall_opt.c:99-122, on device-resident evaluation plans of a GPU target).
 * With refine_gnorm > 0 the evaluations run in float-float until the Riemannian gradient
 * norm falls below refine_gnorm, then in complex128 to the end; refine_gnorm <= 0: complex128
 * throughout.  f_iter [niter+1] gets Re f of every iterate (the last one at vlist_out),
 * prec_iter [niter+1] (may be NULL) the precision each was evaluated in.
 * --------------------------------------------------------------------------------- */
int mg_optimize_brickwall(void* target, const struct matchgate vlist0[], int nlayers, int nqubits, const int* perms[],
                          const struct rtr_params* params, int niter, double refine_gnorm, double f_iter[], int prec_iter[],
                          struct matchgate vlist_out[]);
/* The same fit with one parameter block per gate of a general circuit (gates0 on wires
 * [2 ngates], 8 ngates real parameters; the per-gate Riemannian gradient and Hessian of
 * matchgate_circuit_unitary_target_gradient_vector_hessian_matrix), retraction per gate.
 * The reference optimises per layer only; this is the per-gate extension of that loop. */
int mg_optimize_circuit(void* target, const struct matchgate gates0[], int ngates, const int wires[], int nqubits,
                        const struct rtr_params* params, int niter, double refine_gnorm, double f_iter[], int prec_iter[],
                        struct matchgate gates_out[]);

/* ---------------------------------------------------------------------------------
 * Target construction (the reference builds its benchmark targets in Python,
 * benchmark_hpc/spl_hubbard1d_bench_init.py:24-118, test/rqcopt_matfree/splitting_method.py:
 * 161-193): the spinful 1-D Fermi-Hubbard model on nsites sites (2 nsites qubits,
 * interleaved spins, Jordan-Wigner, open chain), H = U sum n_up n_down - J sum hops, as a
 * Suzuki product formula of even order (2, 4, ...) with nsteps steps over time t, built
 * from on-site phases, hopping matchgates and fermionic swaps.
 * mg_hubbard_trotter_circuit writes the gates and wires when capacity suffices and returns
 * the gate count (< 0 on bad arguments); mg_target_hubbard returns a GPU target of it.
 * --------------------------------------------------------------------------------- */
int mg_hubbard_trotter_circuit(int nsites, double J, double U, double t, int nsteps, int order,
                               struct matchgate gates[], int wires[], int capacity);
void* mg_target_hubbard(int nsites, double J, double U, double t, int nsteps, int order);
/* The spinless chain of the reference's published benchmark: L sites on a ring (periodic
 * wiring), h = -J (|01><10| + |10><01|) + g |11><11| per bond, even and odd bonds as the two
 * terms, as a brickwall with one matchgate per layer (exp(-i tau h) on all L/2 pairs of the
 * layer's permutation: identity for even bonds, shifted by one for odd bonds), neighbouring
 * layers of one term merged.  mg_spinless_hubbard_brickwall writes ulist[n] and the
 * permutations perms[n * L] (row l = layer l) when capacity >= n and returns the layer count
 * n (< 0 on bad arguments); mg_target_spinless_hubbard returns a GPU target of it (12 steps
 * of order 6 at L=16 give the 601-layer target of the published runs). */
int mg_spinless_hubbard_brickwall(int L, double J, double g, double t, int nsteps, int order,
                                  struct matchgate ulist[], int perms[], int capacity);
void* mg_target_spinless_hubbard(int L, double J, double g, double t, int nsteps, int order);

/* ---------------------------------------------------------------------------------
 * Batches: f and the layer gradients of many independent brickwall fits at once, each
 * against its own GPU circuit target (mg_target_circuit / mg_target_brickwall), any
 * even qubit count and depth.  One persistent launch per phase covers every instance:
 * columns are cut into work items of similar cost, taken largest first by all blocks,
 * and the whole launch sequence is captured into a CUDA graph on the first run and
 * replayed after.  Each instance's target tile size is chosen at creation by timing
 * the candidates (2^10 .. 2^12 amplitudes) on a sample of its columns (tune != 0).
 * Results equal those of one-instance evaluations up to summation order
 * (deterministic from run to run).  Precision: the one set when the batch is created.
 * --------------------------------------------------------------------------------- */
typedef struct mg_batch mg_batch;
mg_batch* mg_batch_create(int n, void* const targets[], const struct matchgate* const vlists[], const int nlayers[],
                          const int* const* const perms[], const int nqubits[], int tune);
int mg_batch_set_gates(mg_batch* batch, int i, const struct matchgate vlist[]);
int mg_batch_run(mg_batch* batch);
/* any output may be NULL: f, dvlist [nlayers_i] (as matchgate_brickwall_unitary_target_and_gradient),
 * grad_vec [8 nlayers_i] (Riemannian, as the projected gradient) */
int mg_batch_results(mg_batch* batch, int i, numeric* fval, struct matchgate dvlist[], double* grad_vec);
/* the tuned target tile bits, the target's passes per column and the instance's work items */
int mg_batch_info(mg_batch* batch, int i, int* target_tile_bits, int* target_passes, int* items);
/* GPU time of `steps` graph replays (CUDA events), L2 flushed between them if asked */
double mg_batch_time_ms(mg_batch* batch, int steps, int flush_l2);
void mg_batch_free(mg_batch* batch);

/* ---------------------------------------------------------------------------------
 * Request server (no reference counterpart): evaluations submitted from any thread and
 * served by one worker thread with continuous batching.  Each step takes every queued
 * request whose device workspace estimate fits what is left of the HBM budget (a later
 * request may pass one that does not fit yet; one that can never fit fails with -6),
 * runs all f / gradient requests of the step as one batch (as mg_batch_*), then the
 * Hessian and trust-region-step requests on cached evaluation plans.  Requests that
 * arrive during a step join the next one.  Precision: the library's current one.
 * --------------------------------------------------------------------------------- */
enum { MG_REQ_TARGET = 0, MG_REQ_GRADIENT = 1, MG_REQ_HESSIAN = 2, MG_REQ_TRSTEP = 3 };
typedef struct
{
	int kind;                          /* MG_REQ_* */
	void* target;                      /* GPU target (mg_target_*) on nqubits qubits */
	int nqubits, nlayers;
	const struct matchgate* vlist;     /* [nlayers], copied at submission */
	const int* perms;                  /* [nlayers][nqubits] row-major, copied */
	double radius;                     /* MG_REQ_TRSTEP: trust radius */
} mg_request;
typedef struct mg_server mg_server;
mg_server* mg_server_create(size_t hbm_budget_bytes, int max_batch);
/* returns the request id (>= 0) or an error code (< 0) */
long mg_server_submit(mg_server* server, const mg_request* request);
/* 1 when request id has completed, 0 while it is queued or running */
int mg_server_done(mg_server* server, long id);
/* block until request id completes; its status (0 or an error code) */
int mg_server_wait(mg_server* server, long id);
/* wait, then copy the results (any pointer may be NULL): f (Re f for a trust-region step,
 * at the returned point), grad_vec [8 nlayers] and H [(8 nlayers)^2] (Riemannian, at the
 * request's input point), vlist [nlayers] (a trust-region step's new point: the
 * retracted step when accepted, else the input), the new radius and acceptance,
 * times {submitted, started, completed} in seconds of CLOCK_MONOTONIC, and the step
 * that served it */
int mg_server_result(mg_server* server, long id, numeric* fval, double* grad_vec, double* H, struct matchgate vlist[],
                     double* radius, int* accepted, double times[3], long* step);
/* steps run, requests served in batches, largest budget in use by one step (bytes) */
void mg_server_stats(mg_server* server, long* steps, long* batched, size_t* peak_bytes);
/* serves what is queued, stops the worker and frees everything */
void mg_server_free(mg_server* server);

/* ---------------------------------------------------------------------------------
 * Results the reference computes only inside larger calls
 * --------------------------------------------------------------------------------- */

/* f and the Riemannian gradient vector grad_vec[8*nlayers] (the conjugated,
 * tangent-projected layer gradients of src/matchgate_target.c:903-908) without a
 * Hessian; the reference names this entry point in src/mg_brickwall_opt.c:47. */
int matchgate_brickwall_unitary_target_and_projected_gradient(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, double* grad_vec);

/* Per-gate Hessian of a general circuit: hess is (8*ngates)^2 complex, row g*8+x,
 * column h*8+y (x, y: 0..3 center, 4..7 corner), same conventions as the per-layer
 * Hessian of matchgate_brickwall_unitary_target_gradient_hessian. */
int matchgate_circuit_unitary_target_gradient_hessian(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits,
	numeric* fval, struct matchgate dgates[], numeric* hess);

/* Per-gate Riemannian forms of a general circuit: grad_vec [8 ngates] and H [(8 ngates)^2]
 * (row-major, H[(g*8+x)*m + h*8+y]), the projection of the reference's per-layer
 * matchgate_brickwall_unitary_target_gradient_vector_hessian_matrix (src/matchgate_target.c:
 * 877-973) applied with one block per gate: gradient conjugated and mapped by
 * tangent_matchgate_to_real, Hessian blocks contracted with real_to_tangent unit vectors,
 * conjugated, projected, with the -1/2 (Z dV^dagger V + V dV^dagger Z) term on diagonal
 * blocks.  Summing the blocks of the gates of each layer gives the per-layer forms. */
int matchgate_circuit_unitary_target_and_projected_gradient(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits,
	numeric* fval, double* grad_vec);
int matchgate_circuit_unitary_target_gradient_vector_hessian_matrix(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits,
	numeric* fval, double* grad_vec, double* H);

/* Partial traces over the basis columns b in [col_begin, col_end): the column range
 * the reference gives each MPI rank (benchmark_hpc/benchmark_mpi.c:26-45).  Summing
 * the results of disjoint ranges gives the full trace. */
int mg_brickwall_target_and_gradient_columns(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	long col_begin, long col_end, numeric* fval, struct matchgate dvlist[]);

/* ---------------------------------------------------------------------------------
 * Device-resident evaluation plans: build once, then re-evaluate with new gates
 * without re-planning.  `what` is MG_EVAL_TARGET, MG_EVAL_GRADIENT or
 * MG_EVAL_HESSIAN (| MG_EVAL_TI for the translation-invariant Hessian).
 * mg_plan_run leaves the results on the GPU; mg_plan_results copies them out.
 * --------------------------------------------------------------------------------- */
enum { MG_EVAL_TARGET = 0, MG_EVAL_GRADIENT = 1, MG_EVAL_HESSIAN = 2, MG_EVAL_TI = 4 };
typedef struct mg_plan mg_plan;
mg_plan* mg_plan_brickwall(linear_func ufunc, void* udata, const struct matchgate vlist[], int nlayers, int nqubits,
	const int* perms[], int what);
/* a plan of a general circuit with one parameter block per gate (what: TARGET, GRADIENT or
 * HESSIAN; mg_plan_set_gates takes the ngates gates, the results are per gate) */
mg_plan* mg_plan_circuit(linear_func ufunc, void* udata, const struct matchgate gates[], int ngates, const int wires[],
	int nqubits, int what);
int mg_plan_set_gates(mg_plan* plan, const struct matchgate vlist[]);
int mg_plan_run(mg_plan* plan);
/* any output pointer may be NULL; grad_vec/H are the projected (Riemannian) forms */
int mg_plan_results(mg_plan* plan, numeric* fval, struct matchgate dvlist[], numeric* hess, double* grad_vec, double* H);
void mg_plan_free(mg_plan* plan);
/* GPU time of `steps` back-to-back mg_plan_run calls measured with CUDA events on the
 * library's stream; when flush_l2 != 0 a buffer larger than L2 is written between
 * runs, outside the timed intervals.  Returns the summed milliseconds (< 0 on error). */
double mg_plan_time_ms(mg_plan* plan, int steps, int flush_l2);
/* The target-sweep kernel launches inside the last mg_plan_time_ms call (circuit
 * targets): their number and summed duration from CUDA events around each launch. */
int mg_plan_target_kernel_ms(mg_plan* plan, double* ms, long* launches);
/* The target sweep a plan runs: cfg[0] = 0 (no GPU sweep: dense target or host map), 1 (every
 * amplitude) or 2 (weight-restricted); cfg[1] its tile bits; cfg[2] threads per block (as
 * MG_OPT_TARGET_TUNE chose them); cfg[3] live quartets per thread and iteration
 * (weight-restricted) or basis columns per block (every amplitude). */
int mg_plan_target_config(const mg_plan* plan, int cfg[4]);
/* Number of kernels this library has launched since it was loaded. */
long mg_launch_count(void);
/* Peak FP32 FMA rate of this GPU, measured by a dependent-FMA kernel of this library
 * (GFLOP/s, 2 flops per FMA); used as the roofline denominator of the FP32 pipe. */
double mg_measure_fp32_peak_gflops(void);
double mg_measure_fp64_peak_gflops(void);

/* ---------------------------------------------------------------------------------
 * Allocation-free evaluation.  No counterpart in the reference.
 *
 * For callers that cannot allocate GPU memory while they run -- a host that hands all
 * device memory to its own pool allocator up front, a real-time loop where the implicit
 * synchronisation of cudaMalloc/cudaFree is not acceptable, or a process whose memory
 * budget is fixed at start-up.  Computes, in complex128, f = -tr(U^dagger W) and the raw
 * (holomorphic, unprojected) gradient of f with respect to each layer's shared gate, summed
 * over the layer's gates, for a brickwall W (vlist, perms: every perms[i] a permutation of
 * the qubits) against a target U given as a gate list (ugates on uwires[2g], uwires[2g+1]).
 * It calls no cudaMalloc, cudaFree or other allocating routine, on the device or the host:
 * all workspace lives in one fixed array that every GPU loading this library reserves
 * until the process exits (about 35 MB; one copy per process and GPU).  Limits: even
 * 4 <= nqubits <= 10, nlayers * nqubits / 2 <= 64 fitted gates, ungates <= 4096; larger
 * sizes and invalid wirings are rejected with MG_ERR_ARG (-6) and a message.  The first
 * call on a device looks up the array's device address; make that first call before any
 * stream capture.  All calls of a process share the array, which keeps the last call's
 * contents (the library clears what must start at zero).  The library's lock serialises
 * the calls and each call waits for its GPU work before it returns, so two calls never
 * overlap on the GPU; GPU work of two calls that did overlap would race on the array. */
int mg_noalloc_brickwall_target_and_gradient(const struct matchgate ugates[], int ungates, const int uwires[],
	const struct matchgate vlist[], int nlayers, int nqubits, const int* perms[], numeric* fval, struct matchgate dvlist[]);

#ifdef __cplusplus
}
#endif
