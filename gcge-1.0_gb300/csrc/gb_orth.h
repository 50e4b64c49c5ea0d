/*
 * gb_orth.h -- Cholesky-QR orthonormalisation workspace and entry, shared by
 * the ABI (gb_api.cu) and the host driver (gb_solver.c).
 */
#ifndef GB_ORTH_H
#define GB_ORTH_H

#include "gb_internal.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    gcge_gpu_ctx *ctx;         /* owner of the blocks (its block cache) */
    int max_width, max_start;
    size_t g_cap;    /* doubles in G */
    double *T1;      /* n x ld1 block: B*W and the re-combined columns */
    long ld1;
    double *G;       /* Gram blocks: (max_start + max_width) x max_width */
    double *Tm;      /* max_width^2 coefficient matrix */
    double *Cm;      /* (max_start + max_width) x max_width recombination coefficients */
    double *chol_work;
    double *small;   /* norms */
    int *kept_dev;
    double *ev_work; /* eigensolve of a max_width Gram (w_orth_type cbgs / scbgs) */
    double *ev_val;
    int *ev_info;
} gb_orth_ws;

/* W-orthonormalisation variants (w_orth_type, src/gcge_eigsol.c:448-472) */
enum { GB_ORTH_MULTI = 0, GB_ORTH_CBGS = 1, GB_ORTH_SCBGS = 2, GB_ORTH_GS = 3 };
int gb_orth_kind(const char *w_orth_type);

int  gb_orth_ws_alloc(gcge_gpu_ctx *ctx, gb_orth_ws *ws, int n, int max_width, int max_start);
void gb_orth_ws_free(gb_orth_ws *ws);

/* B-orthonormalise V[:, start:*end) (row-major block, ld ldv) against
 * V[:, 0:start) and itself: up to max_reorth_time block projection passes (a
 * third only when the second still removed more than 1e-10 of the first), then
 * Cholesky-QR twice with deflation; kept columns are packed at start, *end
 * shrinks by the number dropped. With two projection passes, the first
 * Cholesky-QR reuses the second pass's B product (see gb_api.cu). */
int gb_orthonormalize(gcge_gpu_ctx *ctx, int n, double *V, long ldv, int start, int *end,
                      const gcge_gpu_mat *B, int max_reorth_time, double zero_tol, gb_orth_ws *ws);

/* the same contract by the variant `kind`: GB_ORTH_MULTI is gb_orthonormalize;
 * CBGS two block projection passes, then W <- W Q diag(theta)^-1/2 from the
 * eigenpairs (theta, Q) of W^T B W, dropping theta below the zero tolerance
 * (GCGE_CBOrthonormalization, src/gcge_orthogonal.c:755-964); SCBGS the same
 * with the eigenvalue step repeated once to repair its rounding
 * (GCGE_SCBOrthonormalization, :967-1279); GS column by column, two projections
 * of each column against every column before it, then its B-norm
 * (GCGE_BOrthonormalization :352-528 and GCGE_Orthonormalization :112-305). */
int gb_orthonormalize_kind(gcge_gpu_ctx *ctx, int n, double *V, long ldv, int start, int *end,
                           const gcge_gpu_mat *B, int max_reorth_time, double zero_tol, gb_orth_ws *ws, int kind);

/* column-major host n x k  <->  row-major device block columns */
int gb_upload_cols(gcge_gpu_ctx *ctx, int n, int k, const double *host, double *d, long ld);
int gb_download_cols(gcge_gpu_ctx *ctx, int n, int k, const double *d, long ld, double *host);

#ifdef __cplusplus
}
#endif
#endif
