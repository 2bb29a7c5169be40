/*
 * Host ABI of the matchgate algebra (reference src/matchgate.c).  The arithmetic is
 * the shared FP64 code of mg_algebra.h, which the GPU kernels (projection,
 * retraction) compile from the same source; retract_matchgate runs on the GPU.
 */
#include <stdio.h>
#include <string.h>

#include "matchgate.h"
#include "../mg_internal.h"

#define G(p)  ((mgg*)(p))
#define CG(p) ((const mgg*)(p))
#define M2(p) ((mgc*)(p)->data)
#define CM2(p) ((const mgc*)(p)->data)

void compare_matchgate_arrays(const struct matchgate* m, const struct matchgate* n, int d)
{
	printf("\n");
	for (int i = 0; i < d; i++)
	{
		printf("\nMatchgate %d:\n", i);
		for (int k = 0; k < 4; k++)
			printf("Center %d: %lf + %lfi             %lf + %lfi\n", k, creal(m[i].center_block.data[k]), cimag(m[i].center_block.data[k]),
				creal(n[i].center_block.data[k]), cimag(n[i].center_block.data[k]));
		for (int k = 0; k < 4; k++)
			printf("Corner %d (%d): %lf + %lfi             %lf + %lfi\n", k, k + 4, creal(m[i].corner_block.data[k]), cimag(m[i].corner_block.data[k]),
				creal(n[i].corner_block.data[k]), cimag(n[i].corner_block.data[k]));
	}
}

void zero_mat2x2(struct mat2x2* a) { memset(a->data, 0, sizeof(a->data)); }
void identity_mat2x2(struct mat2x2* a) { zero_mat2x2(a); a->data[0] = 1; a->data[3] = 1; }
void zero_matchgate(struct matchgate* a) { mgg_zero(G(a)); }
void identity_matchgate(struct matchgate* a) { mgg_identity(G(a)); }
void scale_matchgate(struct matchgate* restrict a, const double x) { mgg_scale(G(a), x); }
void conjugate_matchgate(struct matchgate* a) { mgg_conj(G(a)); }
void add_matchgate(struct matchgate* restrict a, const struct matchgate* restrict b) { mgg_add(G(a), CG(b)); }
void sub_matchgate(struct matchgate* restrict a, const struct matchgate* restrict b) { mgg_sub(G(a), CG(b)); }
void add_matchgates(const struct matchgate* restrict a, const struct matchgate* restrict b, struct matchgate* restrict c) { *c = *a; mgg_add(G(c), CG(b)); }
void sub_matchgates(const struct matchgate* restrict a, const struct matchgate* restrict b, struct matchgate* restrict c) { *c = *a; mgg_sub(G(c), CG(b)); }
void transpose_matchgate(const struct matchgate* restrict a, struct matchgate* restrict at) { mgg_transpose(CG(a), G(at)); }
void adjoint_matchgate(const struct matchgate* restrict a, struct matchgate* restrict ah) { mgg_adjoint(CG(a), G(ah)); }
void symm_matchgate(const struct matchgate* restrict w, struct matchgate* restrict z) { mgg_symm(CG(w), G(z)); }
void antisymm_matchgate(const struct matchgate* restrict w, struct matchgate* restrict z) { mgg_antisymm(CG(w), G(z)); }
void real_to_antisymm_matchgate(const double* r, struct matchgate* w) { mgg_real_to_antisymm(r, G(w)); }
void antisymm_matchgate_to_real(const struct matchgate* w, double* r) { mgg_antisymm_to_real(CG(w), r); }
void real_to_tangent_matchgate(const double* r, const struct matchgate* restrict v, struct matchgate* restrict z) { mgg_real_to_tangent(r, CG(v), G(z)); }
void tangent_matchgate_to_real(const struct matchgate* restrict v, const struct matchgate* restrict z, double* r) { mgg_tangent_to_real(CG(v), CG(z), r); }
void project_tangent_matchgate(const struct matchgate* restrict u, const struct matchgate* restrict z, struct matchgate* restrict p) { mgg_project_tangent(CG(u), CG(z), G(p)); }
void multiply_mat2x2(const struct mat2x2* a, const struct mat2x2* b, struct mat2x2* restrict c) { mg2_mul(CM2(a), CM2(b), M2(c)); }
void multiply_matchgates(const struct matchgate* restrict a, const struct matchgate* restrict b, struct matchgate* restrict c) { mgg_mul(CG(a), CG(b), G(c)); }
void symmetric_triple_matchgate_product(const struct matchgate* restrict a, const struct matchgate* restrict b, const struct matchgate* restrict c, struct matchgate* restrict ret)
{
	mgg_sym_triple(CG(a), CG(b), CG(c), G(ret));
}

int inverse_mat2x2(const struct mat2x2* restrict a, struct mat2x2* restrict ainv) { return mg2_inv(CM2(a), M2(ainv)); }
int inverse_matchgate(const struct matchgate* restrict a, struct matchgate* restrict ainv) { return mgg_inverse(CG(a), G(ainv)); }
void polar_matchgate_factor(const struct matchgate* restrict a, struct matchgate* restrict u) { mgg_polar(CG(a), G(u)); }

/* v = polar(u (I + A(eta))) on the GPU in FP64 */
void retract_matchgate(const struct matchgate* restrict u, const double* restrict eta, struct matchgate* restrict v)
{
	mgcu_lock();
	int r = mgcu_retract(CG(u), eta, 1, G(v));
	mgcu_unlock();
	if (r) fprintf(stderr, "retract_matchgate failed on the GPU: %s\n", mg_last_error());
}
