/* Compile-time check that GCGE_GPU_OPS_LAYOUT (include/gcge_gb300_ops.h) has the
 * member order, offsets and size of the reference's GCGE_OPS (src/gcge_ops.h:29-215).
 * Compiled by tests/test_abi_cpu.py against the reference headers when present. */
#include <stddef.h>
#include "gcge_ops.h"
#include "gcge_gb300_ops.h"

#define SAME(m) _Static_assert(offsetof(GCGE_OPS, m) == offsetof(GCGE_GPU_OPS_LAYOUT, m), #m)
SAME(VecSetRandomValue); SAME(MatDotVec); SAME(VecAxpby); SAME(VecInnerProd); SAME(VecLocalInnerProd);
SAME(VecCreateByVec); SAME(VecCreateByMat); SAME(VecDestroy); SAME(LinearSolver); SAME(linear_solver_workspace);
SAME(Orthonormalization); SAME(DenseMatCreate); SAME(DenseMatDestroy); SAME(MultiVecCreateByVec);
SAME(MultiVecCreateByMat); SAME(MultiVecCreateByMultiVec); SAME(MultiVecDestroy); SAME(MultiVecSetRandomValue);
SAME(MatDotMultiVec); SAME(MultiVecAxpby); SAME(MultiVecAxpbyColumn); SAME(MultiVecLinearComb);
SAME(MultiVecInnerProd); SAME(MultiVecSwap); SAME(MultiVecPrint); SAME(GetVecFromMultiVec);
SAME(RestoreVecForMultiVec); SAME(SetDirichletBoundary); SAME(DenseMatEigenSolver); SAME(DenseMatDotDenseMat);
SAME(DenseSymMatDotDenseMat); SAME(ArrayDotArray); SAME(ArrayNorm); SAME(ArrayAXPBY); SAME(ArrayCopy);
SAME(ArrayScale);
_Static_assert(sizeof(GCGE_OPS) == sizeof(GCGE_GPU_OPS_LAYOUT), "size");

/* the filler has the signature a GCGE backend init calls with solver->ops */
int fill(GCGE_OPS *ops, gcge_gpu_ctx *ctx) { return GCGE_GPU_SetOps(ctx, ops); }
