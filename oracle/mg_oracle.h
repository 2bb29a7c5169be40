/*
 * ORACLE -- test infrastructure only.
 *
 * A plain-C (C99 complex, OpenMP) restatement of the reference algorithm for the
 * matchgate-brickwall target / gradient / Hessian path of rqcopt_hpc-matchgate.
 * It follows the reference's full-vector, one-basis-column-at-a-time method
 * (no parity-sector compaction, no batching) so that it reproduces the reference's
 * arithmetic; every function cites the reference file:line it restates.
 *
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
 * always as the checker or the timed CPU baseline -- never by the product library.
 *
 * Conventions (reference src/gate.c:581-652, test/rqcopt_matfree/gate.py:19-25):
 *   - qubit 0 is the most significant bit of a basis index;
 *   - a gate on wires (i, j) acts on the local index 2*bit_i + bit_j in the order
 *     |00>, |01>, |10>, |11>; the center block acts on (|01>, |10>) and the corner
 *     block on (|00>, |11>), both row-major 2x2.
 */
#pragma once

#include <complex.h>

typedef double complex orc_c;

/* one parity-preserving two-qubit gate, same memory layout as the reference's
 * struct matchgate (src/matchgate.h:5-14): center block then corner block */
typedef struct { orc_c c[4]; orc_c k[4]; } orc_mg;

/* ---- targets: the caller-supplied linear map U (src/matchgate_target.h:10) ---- */
typedef struct orc_target orc_target;
orc_target* orc_target_hash(int L);                    /* test/test_matchgate_target.c:20-34 */
orc_target* orc_target_dense(const orc_c* U, int L);   /* row-major 2^L x 2^L, test/test_matchgate_target.c:38-47 */
orc_target* orc_target_brickwall(const orc_mg* ulist, int ulayers, const int* uperms, int L); /* test/test_matchgate_target.c:59-66 */
orc_target* orc_target_circuit(const orc_mg* gates, int ngates, const int* wires, int L);
void orc_target_free(orc_target* t);
void orc_target_apply(const orc_target* t, const orc_c* psi, orc_c* out, orc_c* scratch);

/* ---- single-gate kernels (src/gate.c) ---- */
void orc_apply_gate(const orc_mg* g, int i, int j, int L, const orc_c* psi, orc_c* out);
void orc_apply_gate_backward(const orc_mg* g, int i, int j, int L, const orc_c* psi, const orc_c* dpsi_out, orc_c* dpsi, orc_mg* dg);
void orc_apply_gate_array(const orc_mg* g, int i, int j, int L, int nstates, const orc_c* psi, orc_c* out);
void orc_apply_gate_backward_array(const orc_mg* g, int i, int j, int L, int nstates, const orc_c* psi, const orc_c* dpsi_out, orc_mg* dgs);
void orc_apply_placeholder(int i, int j, int L, const orc_c* psi, orc_c* out8);

/* ---- brickwall sweeps (src/matchgate_brickwall.c); perms is nlayers x L, flat ---- */
void orc_brickwall_apply(const orc_mg* vlist, int nlayers, const int* perms, int L, const orc_c* psi, orc_c* out);
void orc_brickwall_forward(const orc_mg* vlist, int nlayers, const int* perms, int L, const orc_c* psi, orc_c* cache, orc_c* out);
void orc_brickwall_backward(const orc_mg* vlist, int nlayers, const int* perms, int L, const orc_c* cache, const orc_c* dpsi_out, orc_c* dpsi, orc_mg* dvlist);
void orc_brickwall_backward_hessian(const orc_mg* vlist, int nlayers, const int* perms, int L, int ti, const orc_c* cache,
	const orc_c* dpsi_out, orc_c* dpsi, orc_mg* dvlist, orc_c* hess);

/* ---- general circuits (src/quantum_circuit.c); wires is 2*ngates ---- */
void orc_circuit_apply(const orc_mg* gates, int ngates, const int* wires, int L, const orc_c* psi, orc_c* out);
void orc_circuit_forward(const orc_mg* gates, int ngates, const int* wires, int L, const orc_c* psi, orc_c* cache, orc_c* out);
void orc_circuit_backward(const orc_mg* gates, int ngates, const int* wires, int L, const orc_c* cache, const orc_c* dpsi_out, orc_c* dpsi, orc_mg* dgates);

/* ---- traces over basis columns b in [col_begin, col_end) (src/matchgate_target.c);
 *      nthreads <= 0 means the OpenMP default; col_end < 0 means all 2^L columns ---- */
int orc_circuit_target(const orc_target* t, const orc_mg* gates, int ngates, const int* wires, int L,
	int nthreads, long col_begin, long col_end, orc_c* fval);
int orc_circuit_target_and_gradient(const orc_target* t, const orc_mg* gates, int ngates, const int* wires, int L,
	int nthreads, long col_begin, long col_end, orc_c* fval, orc_mg* dgates);
int orc_circuit_target_gradient_hessian(const orc_target* t, const orc_mg* gates, int ngates, const int* wires, int L,
	int nthreads, long col_begin, long col_end, orc_c* fval, orc_mg* dgates, orc_c* hess);
int orc_brickwall_target(const orc_target* t, const orc_mg* vlist, int nlayers, const int* perms, int L,
	int nthreads, long col_begin, long col_end, orc_c* fval);
int orc_brickwall_target_and_gradient(const orc_target* t, const orc_mg* vlist, int nlayers, const int* perms, int L,
	int nthreads, long col_begin, long col_end, orc_c* fval, orc_mg* dvlist);
int orc_brickwall_target_gradient_hessian(const orc_target* t, const orc_mg* vlist, int nlayers, const int* perms, int L, int ti,
	int nthreads, long col_begin, long col_end, orc_c* fval, orc_mg* dvlist, orc_c* hess);
int orc_brickwall_projected_gradient(const orc_target* t, const orc_mg* vlist, int nlayers, const int* perms, int L,
	int nthreads, long col_begin, long col_end, orc_c* fval, double* grad_vec);
int orc_brickwall_gradvec_hessmat(const orc_target* t, const orc_mg* vlist, int nlayers, const int* perms, int L, int ti,
	int nthreads, orc_c* fval, double* grad_vec, double* H);

/* ---- matchgate algebra (src/matchgate.c) ---- */
void orc_mg_multiply(const orc_mg* a, const orc_mg* b, orc_mg* c);
void orc_mg_adjoint(const orc_mg* a, orc_mg* ah);
void orc_mg_conj(orc_mg* a);
void orc_mg_symm(const orc_mg* w, orc_mg* z);
void orc_mg_antisymm(const orc_mg* w, orc_mg* z);
void orc_mg_real_to_antisymm(const double* r, orc_mg* w);
void orc_mg_antisymm_to_real(const orc_mg* w, double* r);
void orc_mg_real_to_tangent(const double* r, const orc_mg* v, orc_mg* z);
void orc_mg_tangent_to_real(const orc_mg* v, const orc_mg* z, double* r);
void orc_mg_project_tangent(const orc_mg* u, const orc_mg* z, orc_mg* p);
int orc_mg_inverse(const orc_mg* a, orc_mg* ainv);
void orc_mg_polar(const orc_mg* a, orc_mg* u);
void orc_mg_retract(const orc_mg* u, const double* eta, orc_mg* v);
void orc_project_hessian(const orc_mg* vlist, const orc_mg* dvlist_conj, int nlayers, const orc_c* hess, double* H);

/* ---- trust region (src/trust_region.c) ---- */
int orc_truncated_cg(const double* grad, const double* hess, int n, double radius, int maxiter, double abstol, double reltol, double* z);
void orc_rtr_brickwall(const orc_target* t, const orc_mg* vlist0, int nlayers, const int* perms, int L, int ti, int nthreads,
	int niter, int tcg_maxiter, double rho_trust, double radius_init, double maxradius,
	double* f_iter, orc_c* f_citer, orc_mg* vlist_out);
