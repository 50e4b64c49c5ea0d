// gb_api.cu -- C ABI: context, device CSR matrices, multivectors, block
// operations and the Cholesky-QR orthonormalisation (include/gcge_gb300.h).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cuda_runtime.h>

#include "gb_internal.h"
#include "gb_orth.h"

#define GB_LAUNCH(ctx, kern, grid, block, smem, ...)                                   \
    do {                                                                               \
        kern<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);                 \
        (ctx)->launches++;                                                             \
        int _st = gb_check_launch(ctx);                                                \
        if (_st) return _st;                                                           \
    } while (0)

#define CUDA_TRY(ctx, call)                                                            \
    do {                                                                               \
        if ((call) != cudaSuccess) return gb_fail((ctx), GCGE_GPU_ERR_CUDA);           \
    } while (0)

extern "C" int gb_fail(gcge_gpu_ctx *ctx, int st)
{
    if (ctx && st && !ctx->err) ctx->err = st;
    return st;
}

extern "C" int gb_check_launch(gcge_gpu_ctx *ctx)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        fprintf(stderr, "gcge_gb300: CUDA error %s\n", cudaGetErrorString(e));
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    }
    return GCGE_GPU_OK;
}

static int grow(gcge_gpu_ctx *ctx, double **p, size_t *cap, size_t n, int pinned)
{
    if (*cap >= n) return GCGE_GPU_OK;
    size_t want = n + n / 4 + 1024;
    if (*p) {
        if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
        if (pinned) cudaFreeHost(*p);
        else cudaFree(*p);
        *p = nullptr;
        *cap = 0;
    }
    cudaError_t e = pinned ? cudaMallocHost((void **)p, want * sizeof(double))
                           : cudaMalloc((void **)p, want * sizeof(double));
    if (e != cudaSuccess) {
        *p = nullptr;
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    *cap = want;
    return GCGE_GPU_OK;
}
extern "C" int gb_scratch(gcge_gpu_ctx *ctx, size_t n) { return grow(ctx, &ctx->scratch, &ctx->scratch_cap, n, 0); }
extern "C" int gb_coef(gcge_gpu_ctx *ctx, size_t n) { return grow(ctx, &ctx->coef, &ctx->coef_cap, n, 0); }
extern "C" int gb_pinned(gcge_gpu_ctx *ctx, size_t n) { return grow(ctx, &ctx->pinned, &ctx->pinned_cap, n, 1); }
extern "C" int gb_iscratch(gcge_gpu_ctx *ctx, size_t n)
{
    if (ctx->iscratch_cap >= n) return GCGE_GPU_OK;
    if (ctx->iscratch) {
        if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
        cudaFree(ctx->iscratch);
        ctx->iscratch = nullptr;
        ctx->iscratch_cap = 0;
    }
    const size_t want = n + 1024;
    if (cudaMalloc(&ctx->iscratch, want * sizeof(int)) != cudaSuccess) return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    ctx->iscratch_cap = want;
    return GCGE_GPU_OK;
}

// after a stream synchronisation: GCGE_GPU_ERR_TIMEOUT when a kernel reported
// that one of its bounded waits ran out (its results are then invalid)
extern "C" int gb_check_device_error(gcge_gpu_ctx *ctx)
{
    int h = 0;
    if (cudaMemcpyAsync(&h, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    return h ? gb_fail(ctx, GCGE_GPU_ERR_TIMEOUT) : GCGE_GPU_OK;
}

extern "C" int gb_ozbuf(gcge_gpu_ctx *ctx, size_t bytes)
{
    if (ctx->ozbuf_cap >= bytes) return GCGE_GPU_OK;
    if (ctx->ozbuf) {
        if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
        cudaFree(ctx->ozbuf);
        ctx->ozbuf = nullptr;
        ctx->ozbuf_cap = 0;
    }
    const size_t want = bytes + bytes / 4 + 4096;
    if (cudaMalloc(&ctx->ozbuf, want) != cudaSuccess) {
        ctx->ozbuf = nullptr;
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    ctx->ozbuf_cap = want;
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_SetTensorEmulation(gcge_gpu_ctx *ctx, int on)
{
    if (!ctx) return GCGE_GPU_ERR_ARG;
    ctx->tc = on ? 1 : 0;
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_TestStallTensorWait(gcge_gpu_ctx *ctx, int on)
{
    if (!ctx) return GCGE_GPU_ERR_ARG;
    ctx->tc_stall = on ? 1 : 0;
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_SetPairSpMM(gcge_gpu_ctx *ctx, int on)
{
    if (!ctx) return GCGE_GPU_ERR_ARG;
    ctx->spmm_pair = on ? 1 : 0;
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- context
extern "C" int GCGE_GPU_Init(int device, gcge_gpu_ctx **out)
{
    if (!out) return GCGE_GPU_ERR_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) return GCGE_GPU_ERR_CUDA;
    if (cudaSetDevice(device) != cudaSuccess) return GCGE_GPU_ERR_CUDA;
    gcge_gpu_ctx *c = (gcge_gpu_ctx *)calloc(1, sizeof(gcge_gpu_ctx));
    if (!c) return GCGE_GPU_ERR_NOMEM;
    c->device = device;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (c->num_sms <= 0) c->num_sms = 1;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        free(c);
        return GCGE_GPU_ERR_CUDA;
    }
    c->tc = 1;
    int st = gb_scratch(c, 1 << 20);
    if (!st) st = gb_iscratch(c, 4096);
    if (!st) st = gb_coef(c, 1 << 16);
    if (!st) st = gb_pinned(c, 1 << 16);
    if (!st) st = gb_ozbuf(c, 1 << 20);
    if (!st && (cudaMalloc(&c->dev_err, sizeof(int)) != cudaSuccess ||
                cudaMemsetAsync(c->dev_err, 0, sizeof(int), c->stream) != cudaSuccess ||
                cudaMalloc(&c->dev_pairflag, sizeof(int)) != cudaSuccess ||
                cudaMemsetAsync(c->dev_pairflag, 0, sizeof(int), c->stream) != cudaSuccess))
        st = GCGE_GPU_ERR_NOMEM;
    if (st) {
        GCGE_GPU_Finalize(c);
        return st;
    }
    *out = c;
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- device block cache
// The workspace of a solve (the basis V, scratch blocks, the orthonormalisation
// and block-CG work; several GB at n ~ 1e6) goes back to the context instead of
// cudaFree, so repeated solves on a context reuse it rather than paying
// cudaMalloc/cudaFree of every block each time. Blocks are used on the context's
// stream only, so handing one to a later request is stream-ordered.
extern "C" int gb_dev_alloc(gcge_gpu_ctx *ctx, void **p, size_t bytes)
{
    *p = nullptr;
    if (bytes == 0) bytes = 8;
    int best = -1;
    for (int i = 0; i < ctx->nblk; ++i) {
        const gb_block &b = ctx->blk[i];
        if (!b.used && b.bytes >= bytes && b.bytes <= 2 * bytes && (best < 0 || b.bytes < ctx->blk[best].bytes))
            best = i;
    }
    if (best >= 0) {
        ctx->blk[best].used = 1;
        *p = ctx->blk[best].p;
        return GCGE_GPU_OK;
    }
    void *q = nullptr;
    if (cudaMalloc(&q, bytes) != cudaSuccess) {
        cudaGetLastError();
        // give the unused cached blocks back and try once more
        int k = 0;
        for (int i = 0; i < ctx->nblk; ++i) {
            if (ctx->blk[i].used) ctx->blk[k++] = ctx->blk[i];
            else cudaFree(ctx->blk[i].p);
        }
        ctx->nblk = k;
        if (cudaMalloc(&q, bytes) != cudaSuccess) {
            cudaGetLastError();
            return GCGE_GPU_ERR_NOMEM;
        }
    }
    if (ctx->nblk == ctx->blk_cap) {
        const int nc = ctx->blk_cap ? 2 * ctx->blk_cap : 64;
        gb_block *nb = (gb_block *)realloc(ctx->blk, sizeof(gb_block) * nc);
        if (!nb) {
            cudaFree(q);
            return GCGE_GPU_ERR_NOMEM;
        }
        ctx->blk = nb;
        ctx->blk_cap = nc;
    }
    ctx->blk[ctx->nblk++] = gb_block{q, bytes, 1};
    *p = q;
    return GCGE_GPU_OK;
}

extern "C" void gb_dev_free(gcge_gpu_ctx *ctx, void *p)
{
    if (!p) return;
    for (int i = 0; i < ctx->nblk; ++i)
        if (ctx->blk[i].p == p) {
            ctx->blk[i].used = 0;
            return;
        }
    cudaFree(p);
}

extern "C" int GCGE_GPU_Finalize(gcge_gpu_ctx *ctx)
{
    if (!ctx) return GCGE_GPU_OK;
    cudaStreamSynchronize(ctx->stream);
    for (int i = 0; i < ctx->nblk; ++i) cudaFree(ctx->blk[i].p);
    free(ctx->blk);
    if (ctx->prof_ev) {
        for (int i = 0; i < 2 * GB_PROF_SLOTS; ++i)
            if (ctx->prof_ev[i]) cudaEventDestroy(ctx->prof_ev[i]);
        free(ctx->prof_ev);
        free(ctx->prof_cls);
        free(ctx->prof_bytes);
        free(ctx->prof_flops);
    }
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->iscratch) cudaFree(ctx->iscratch);
    if (ctx->coef) cudaFree(ctx->coef);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->ozbuf) cudaFree(ctx->ozbuf);
    if (ctx->dev_err) cudaFree(ctx->dev_err);
    if (ctx->dev_pairflag) cudaFree(ctx->dev_pairflag);
    if (ctx->pairbuf) cudaFree(ctx->pairbuf);
    cudaStreamDestroy(ctx->stream);
    free(ctx);
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_GetLastError(gcge_gpu_ctx *ctx)
{
    if (!ctx) return GCGE_GPU_ERR_ARG;
    int e = ctx->err;
    ctx->err = 0;
    return e;
}

extern "C" const char *GCGE_GPU_ErrorString(int st)
{
    switch (st) {
    case GCGE_GPU_OK: return "ok";
    case GCGE_GPU_ERR_ARG: return "invalid argument";
    case GCGE_GPU_ERR_CUDA: return "CUDA runtime error";
    case GCGE_GPU_ERR_NOMEM: return "device allocation failed";
    case GCGE_GPU_ERR_CSR: return "malformed CSR matrix";
    case GCGE_GPU_ERR_NONFINITE: return "non-finite value";
    case GCGE_GPU_ERR_BREAKDOWN: return "orthogonalisation lost every column";
    case GCGE_GPU_ERR_EIGSOLVE: return "projected eigensolve failed";
    case GCGE_GPU_ERR_TIMEOUT: return "tensor-core kernel wait timed out";
    case GCGE_GPU_ERR_IO: return "file missing, unreadable, truncated or not CSR";
    default: return "unknown status";
    }
}

extern "C" int GCGE_GPU_Synchronize(gcge_gpu_ctx *ctx)
{
    if (!ctx) return GCGE_GPU_ERR_ARG;
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return gb_check_device_error(ctx);
}

extern "C" long long GCGE_GPU_LaunchCount(const gcge_gpu_ctx *ctx) { return ctx ? ctx->launches : 0; }

// ---------------------------------------------------------------- profiling mode
static int s_prof_open = 0;

static void prof_resolve(gcge_gpu_ctx *ctx)
{
    if (ctx->prof_used <= 0) return;
    cudaEventSynchronize(ctx->prof_ev[2 * ctx->prof_used - 1]);
    for (int i = 0; i < ctx->prof_used; ++i) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ctx->prof_ev[2 * i], ctx->prof_ev[2 * i + 1]) != cudaSuccess) continue;
        const int c = ctx->prof_cls[i];
        ctx->cls_ms[c] += ms;
        ctx->cls_bytes[c] += ctx->prof_bytes[i];
        ctx->cls_flops[c] += ctx->prof_flops[i];
        ctx->cls_launches[c] += 1;
    }
    ctx->prof_used = 0;
}

extern "C" void gb_prof_begin(gcge_gpu_ctx *ctx, int cls, double bytes, double flops)
{
    if (!ctx->prof || !ctx->prof_ev) return;
    if (ctx->prof_used >= GB_PROF_SLOTS) prof_resolve(ctx);
    const int i = ctx->prof_used;
    ctx->prof_cls[i] = cls;
    ctx->prof_bytes[i] = bytes;
    ctx->prof_flops[i] = flops;
    cudaEventRecord(ctx->prof_ev[2 * i], ctx->stream);
    s_prof_open = 1;
}

extern "C" void gb_prof_end(gcge_gpu_ctx *ctx)
{
    if (!s_prof_open) return;
    s_prof_open = 0;
    cudaEventRecord(ctx->prof_ev[2 * ctx->prof_used + 1], ctx->stream);
    ctx->prof_used++;
}

extern "C" int GCGE_GPU_ProfileEnable(gcge_gpu_ctx *ctx, int on)
{
    if (!ctx) return GCGE_GPU_ERR_ARG;
    if (on && !ctx->prof_ev) {
        ctx->prof_ev = (cudaEvent_t *)calloc(2 * GB_PROF_SLOTS, sizeof(cudaEvent_t));
        ctx->prof_cls = (int *)calloc(GB_PROF_SLOTS, sizeof(int));
        ctx->prof_bytes = (double *)calloc(GB_PROF_SLOTS, sizeof(double));
        ctx->prof_flops = (double *)calloc(GB_PROF_SLOTS, sizeof(double));
        if (!ctx->prof_ev || !ctx->prof_cls || !ctx->prof_bytes || !ctx->prof_flops) return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
        for (int i = 0; i < 2 * GB_PROF_SLOTS; ++i)
            if (cudaEventCreate(&ctx->prof_ev[i]) != cudaSuccess) return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    }
    if (!on) prof_resolve(ctx);
    ctx->prof = on ? 1 : 0;
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_ProfileRead(gcge_gpu_ctx *ctx, int nclass, double *ms, long long *launches, double *bytes,
                                    double *flops, int reset)
{
    if (!ctx) return GCGE_GPU_ERR_ARG;
    prof_resolve(ctx);
    for (int c = 0; c < nclass && c < GB_PROF_CLASSES; ++c) {
        if (ms) ms[c] = ctx->cls_ms[c];
        if (launches) launches[c] = ctx->cls_launches[c];
        if (bytes) bytes[c] = ctx->cls_bytes[c];
        if (flops) flops[c] = ctx->cls_flops[c];
    }
    if (reset) {
        memset(ctx->cls_ms, 0, sizeof(ctx->cls_ms));
        memset(ctx->cls_bytes, 0, sizeof(ctx->cls_bytes));
        memset(ctx->cls_flops, 0, sizeof(ctx->cls_flops));
        memset(ctx->cls_launches, 0, sizeof(ctx->cls_launches));
    }
    return GB_PROF_CLASSES;
}

// ---------------------------------------------------------------- matrices
__global__ void k_d2f_vals(long n, const double *a, float *b)
{
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x)
        b[t] = (float)a[t];
}

// structural check of an uploaded CSR matrix: res[0] = 1 if a row pointer
// decreases or a column lies outside [0, n); res[1] = the longest row
__global__ void k_csr_check(int n, int nnz, const int *__restrict__ rp, const int *__restrict__ ci, int *res)
{
    int bad = 0, mr = 0;
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int len = rp[i + 1] - rp[i];
        bad |= len < 0;
        mr = max(mr, len);
    }
    for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += stride) {
        const int c = ci[e];
        bad |= c < 0 || c >= n;
    }
    for (int o = 16; o; o >>= 1) {
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
        mr = max(mr, __shfl_xor_sync(0xffffffffu, mr, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (bad) atomicOr(res, 1);
        atomicMax(res + 1, mr);
    }
}

// Rows with more than thresh entries, longest first (ties by row), written to
// out (room for every row); returns their count and their entries in *nnz_long.
// Host only (internal, not part of the public interface; the CPU tests call it).
extern "C" int gb_long_rows_host(int n, const int *rowptr, int thresh, int *out, long *nnz_long)
{
    int cnt = 0;
    long nz = 0;
    for (int r = 0; r < n; ++r) {
        const int len = rowptr[r + 1] - rowptr[r];
        if (len > thresh) {
            out[cnt++] = r;
            nz += len;
        }
    }
    std::sort(out, out + cnt, [rowptr](int a, int b) {
        const int la = rowptr[a + 1] - rowptr[a], lb = rowptr[b + 1] - rowptr[b];
        return la != lb ? la > lb : a < b;
    });
    if (nnz_long) *nnz_long = nz;
    return cnt;
}

// The rows longer than GB_LONG_ROW, listed on the device for the FP32 block-CG
// SpMM, which gives each of them a whole block (a grid-stride row split would
// leave a power-law graph's hub rows, up to thousands of entries, to one lane
// group). Called after the structure check, so the lengths are valid.
static int gb_list_long_rows(gcge_gpu_ctx *ctx, gcge_gpu_mat *A, const int *rowptr)
{
    long cnt = 0;
    for (int r = 0; r < A->n; ++r)
        if (rowptr[r + 1] - rowptr[r] > GB_LONG_ROW) ++cnt;
    if (!cnt) return 0;
    int *h = (int *)malloc(sizeof(int) * cnt);
    if (!h) return 1;
    long nz = 0;
    gb_long_rows_host(A->n, rowptr, GB_LONG_ROW, h, &nz);
    int rc = cudaMalloc(&A->lrows, sizeof(int) * cnt) != cudaSuccess ||
             cudaMemcpyAsync(A->lrows, h, sizeof(int) * cnt, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
             cudaStreamSynchronize(ctx->stream) != cudaSuccess;
    free(h);
    if (rc) return 1;
    A->nlong = (int)cnt;
    A->nnz_long = nz;
    return 0;
}

// The structure is checked on the device after the upload (a host loop over
// the column indices cost ~20 ms per 40 M entries, on the path of every
// host-buffer solve); the result is read back with the creation's final sync.
extern "C" int GCGE_GPU_MatCreate(gcge_gpu_ctx *ctx, int n, const int *rowptr, const int *col, const double *val,
                                  int keep_fp32, gcge_gpu_mat **out)
{
    if (!ctx || !out || n <= 0 || !rowptr || (!col && rowptr[n] > 0) || (!val && rowptr[n] > 0))
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    *out = nullptr;
    if (rowptr[0] != 0 || rowptr[n] < 0) return gb_fail(ctx, GCGE_GPU_ERR_CSR);
    const int nnz = rowptr[n];
    gcge_gpu_mat *A = (gcge_gpu_mat *)calloc(1, sizeof(gcge_gpu_mat));
    if (!A) return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    A->ctx = ctx;
    A->n = n;
    A->nnz = nnz;
    size_t nz = nnz > 0 ? (size_t)nnz : 1;
    int *chk = nullptr;
    if (cudaMalloc(&A->rp, sizeof(int) * (n + 1)) != cudaSuccess || cudaMalloc(&A->ci, sizeof(int) * nz) != cudaSuccess ||
        cudaMalloc(&A->v, sizeof(double) * nz) != cudaSuccess ||
        (keep_fp32 && cudaMalloc(&A->v32, sizeof(float) * nz) != cudaSuccess) ||
        cudaMalloc(&chk, 2 * sizeof(int)) != cudaSuccess) {
        if (chk) cudaFree(chk);
        GCGE_GPU_MatDestroy(A);
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    int h[2] = {0, 0};
    if (cudaMemsetAsync(chk, 0, 2 * sizeof(int), ctx->stream) != cudaSuccess ||
        cudaMemcpyAsync(A->rp, rowptr, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        (nnz && cudaMemcpyAsync(A->ci, col, sizeof(int) * nnz, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess) ||
        (nnz && cudaMemcpyAsync(A->v, val, sizeof(double) * nnz, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)) {
        cudaFree(chk);
        GCGE_GPU_MatDestroy(A);
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    }
    k_csr_check<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(n, nnz, A->rp, A->ci, chk);
    ctx->launches++;
    if (keep_fp32 && nnz) {
        k_d2f_vals<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(nnz, A->v, A->v32);
        ctx->launches++;
    }
    if (gb_check_launch(ctx) || cudaMemcpyAsync(h, chk, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        cudaFree(chk);
        GCGE_GPU_MatDestroy(A);
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    }
    cudaFree(chk);
    if (h[0]) {
        GCGE_GPU_MatDestroy(A);
        return gb_fail(ctx, GCGE_GPU_ERR_CSR);
    }
    A->max_row_nnz = h[1];
    if (keep_fp32 && h[1] > GB_LONG_ROW && gb_list_long_rows(ctx, A, rowptr)) {
        GCGE_GPU_MatDestroy(A);
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    *out = A;
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_MatSetValues(gcge_gpu_mat *A, const double *val)
{
    if (!A || !val) return GCGE_GPU_ERR_ARG;
    gcge_gpu_ctx *ctx = A->ctx;
    if (!A->nnz) return GCGE_GPU_OK;
    CUDA_TRY(ctx, cudaMemcpyAsync(A->v, val, sizeof(double) * A->nnz, cudaMemcpyHostToDevice, ctx->stream));
    if (A->dinv || A->vpair) {             // the Jacobi diagonal and the pairs follow the values
        cudaStreamSynchronize(ctx->stream);
        if (A->dinv) cudaFree(A->dinv);
        if (A->dinv32) cudaFree(A->dinv32);
        if (A->vpair) cudaFree(A->vpair);
        if (A->pair_meta) cudaFree(A->pair_meta);
        A->dinv = nullptr;
        A->dinv32 = nullptr;
        A->vpair = nullptr;
        A->pair_meta = nullptr;
    }
    if (A->v32) {
        k_d2f_vals<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(A->nnz, A->v, A->v32);
        ctx->launches++;
        if (gb_check_launch(ctx)) return GCGE_GPU_ERR_CUDA;
    }
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_MatDestroy(gcge_gpu_mat *A)
{
    if (!A) return GCGE_GPU_OK;
    if (A->ctx) cudaStreamSynchronize(A->ctx->stream);
    if (A->rp) cudaFree(A->rp);
    if (A->ci) cudaFree(A->ci);
    if (A->v) cudaFree(A->v);
    if (A->v32) cudaFree(A->v32);
    if (A->dinv) cudaFree(A->dinv);
    if (A->dinv32) cudaFree(A->dinv32);
    if (A->vpair) cudaFree(A->vpair);
    if (A->pair_meta) cudaFree(A->pair_meta);
    if (A->lrows) cudaFree(A->lrows);
    free(A);
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_MatGetSize(const gcge_gpu_mat *A, int *n, int *nnz)
{
    if (!A) return GCGE_GPU_ERR_ARG;
    if (n) *n = A->n;
    if (nnz) *nnz = A->nnz;
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- multivectors
extern "C" int GCGE_GPU_MultiVecCreate(gcge_gpu_ctx *ctx, int n, int ncols, gcge_gpu_mv **out)
{
    if (!ctx || !out || n <= 0 || ncols <= 0) return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    gcge_gpu_mv *m = (gcge_gpu_mv *)calloc(1, sizeof(gcge_gpu_mv));
    if (!m) return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    m->ctx = ctx;
    m->n = n;
    m->ncols = ncols;
    m->ld = (ncols + 1) & ~1;
    if (cudaMalloc(&m->d, sizeof(double) * (size_t)n * m->ld) != cudaSuccess) {
        free(m);
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    if (cudaMemsetAsync(m->d, 0, sizeof(double) * (size_t)n * m->ld, ctx->stream) != cudaSuccess) {
        cudaFree(m->d);
        free(m);
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    }
    *out = m;
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_MultiVecDestroy(gcge_gpu_mv *m)
{
    if (!m) return GCGE_GPU_OK;
    cudaStreamSynchronize(m->ctx->stream);
    cudaFree(m->d);
    free(m);
    return GCGE_GPU_OK;
}

// column-major (ld n) <-> row-major block columns, through a tiled transpose
__global__ void k_cm_to_rm(int n, int k, const double *__restrict__ src, double *__restrict__ dst, long ld)
{
    __shared__ double t[32][33];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int c = c0 + q, r = r0 + threadIdx.x;
        t[q][threadIdx.x] = (r < n && c < k) ? src[(long)c * n + r] : 0.0;
    }
    __syncthreads();
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int r = r0 + q, c = c0 + threadIdx.x;
        if (r < n && c < k) dst[(long)r * ld + c] = t[threadIdx.x][q];
    }
}
__global__ void k_rm_to_cm(int n, int k, const double *__restrict__ src, long ld, double *__restrict__ dst)
{
    __shared__ double t[32][33];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int r = r0 + q, c = c0 + threadIdx.x;
        t[q][threadIdx.x] = (r < n && c < k) ? src[(long)r * ld + c] : 0.0;
    }
    __syncthreads();
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int c = c0 + q, r = r0 + threadIdx.x;
        if (r < n && c < k) dst[(long)c * n + r] = t[threadIdx.x][q];
    }
}

extern "C" int gb_upload_cols(gcge_gpu_ctx *ctx, int n, int k, const double *host, double *d, long ld)
{
    if (n <= 0 || k <= 0) return GCGE_GPU_OK;
    double *stage = nullptr;
    CUDA_TRY(ctx, cudaMalloc(&stage, sizeof(double) * (size_t)n * k));
    if (cudaMemcpyAsync(stage, host, sizeof(double) * (size_t)n * k, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess) {
        cudaFree(stage);
        return gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    }
    dim3 grid((n + 31) / 32, (k + 31) / 32), block(32, 8);
    k_cm_to_rm<<<grid, block, 0, ctx->stream>>>(n, k, stage, d, ld);
    ctx->launches++;
    int st = gb_check_launch(ctx);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(stage);
    return st;
}

extern "C" int gb_download_cols(gcge_gpu_ctx *ctx, int n, int k, const double *d, long ld, double *host)
{
    if (n <= 0 || k <= 0) return GCGE_GPU_OK;
    double *stage = nullptr;
    CUDA_TRY(ctx, cudaMalloc(&stage, sizeof(double) * (size_t)n * k));
    dim3 grid((n + 31) / 32, (k + 31) / 32), block(32, 8);
    k_rm_to_cm<<<grid, block, 0, ctx->stream>>>(n, k, d, ld, stage);
    ctx->launches++;
    int st = gb_check_launch(ctx);
    if (!st && cudaMemcpyAsync(host, stage, sizeof(double) * (size_t)n * k, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
        st = gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) st = gb_fail(ctx, GCGE_GPU_ERR_CUDA);
    cudaFree(stage);
    return st;
}

static int range_ok(const gcge_gpu_mv *m, int c0, int k) { return m && c0 >= 0 && k >= 0 && c0 + k <= m->ncols; }

extern "C" int GCGE_GPU_MultiVecUpload(gcge_gpu_mv *m, int col0, int ncols, const double *host)
{
    if (!range_ok(m, col0, ncols) || (!host && ncols)) return gb_fail(m ? m->ctx : nullptr, GCGE_GPU_ERR_ARG);
    return gb_upload_cols(m->ctx, m->n, ncols, host, m->d + col0, m->ld);
}

extern "C" int GCGE_GPU_MultiVecDownload(const gcge_gpu_mv *m, int col0, int ncols, double *host)
{
    if (!range_ok(m, col0, ncols) || (!host && ncols)) return gb_fail(m ? m->ctx : nullptr, GCGE_GPU_ERR_ARG);
    return gb_download_cols(m->ctx, m->n, ncols, m->d + col0, m->ld, host);
}

extern "C" int GCGE_GPU_MultiVecSetRandomValue(gcge_gpu_mv *m, int start, int nvec, unsigned long long seed)
{
    if (!range_ok(m, start, nvec)) return gb_fail(m ? m->ctx : nullptr, GCGE_GPU_ERR_ARG);
    return gb_fill_random(m->ctx, m->n, nvec, m->d + start, m->ld, start, seed);
}

// ---------------------------------------------------------------- block operations
extern "C" int GCGE_GPU_MatDotMultiVec(const gcge_gpu_mat *A, const gcge_gpu_mv *x, gcge_gpu_mv *y, const int *start,
                                       const int *end)
{
    if (!A || !x || !y || !start || !end) return GCGE_GPU_ERR_ARG;
    const int k = end[0] - start[0];
    if (k != end[1] - start[1] || !range_ok(x, start[0], k) || !range_ok(y, start[1], k) || x->n != A->n ||
        y->n != A->n)
        return gb_fail(A->ctx, GCGE_GPU_ERR_ARG);
    if (x->d == y->d && k > 0) {
        // in-place ranges overlap only if they intersect
        if (!(start[0] + k <= start[1] || start[1] + k <= start[0])) return gb_fail(A->ctx, GCGE_GPU_ERR_ARG);
    }
    return gb_spmm(A->ctx, A, x->d + start[0], x->ld, y->d + start[1], y->ld, k, 1.0, nullptr, 0.0, nullptr);
}

extern "C" int GCGE_GPU_MultiVecAxpby(double a, const gcge_gpu_mv *x, double b, gcge_gpu_mv *y, const int *start,
                                      const int *end)
{
    if (!x || !y || !start || !end) return GCGE_GPU_ERR_ARG;
    const int k = end[0] - start[0];
    if (!range_ok(x, start[0], k) || !range_ok(y, start[1], k) || x->n != y->n) return gb_fail(x->ctx, GCGE_GPU_ERR_ARG);
    return gb_axpby(x->ctx, x->n, k, a, x->d + start[0], x->ld, b, y->d + start[1], y->ld);
}

extern "C" int GCGE_GPU_MultiVecLinearComb(const gcge_gpu_mv *x, gcge_gpu_mv *y, const int *start, const int *end,
                                           const double *a, int lda)
{
    if (!x || !y || !start || !end) return GCGE_GPU_ERR_ARG;
    gcge_gpu_ctx *ctx = x->ctx;
    const int k1 = end[0] - start[0], k2 = end[1] - start[1];
    if (!range_ok(x, start[0], k1) || !range_ok(y, start[1], k2) || x->n != y->n || (k1 > 0 && lda < k1) || (!a && k1 && k2))
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (x->d == y->d && k1 > 0 && k2 > 0 && !(start[0] + k1 <= start[1] || start[1] + k2 <= start[0]))
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (k2 <= 0) return GCGE_GPU_OK;
    int st = gb_coef(ctx, (size_t)k1 * k2 + 1);
    if (st) return st;
    // compact the coefficients (k1 x k2, ld k1) on the host side of the copy
    if ((st = gb_pinned(ctx, (size_t)k1 * k2 + 1))) return st;
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    for (int j = 0; j < k2; ++j) memcpy(ctx->pinned + (size_t)j * k1, a + (size_t)j * lda, sizeof(double) * k1);
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->coef, ctx->pinned, sizeof(double) * (size_t)k1 * k2, cudaMemcpyHostToDevice,
                                  ctx->stream));
    st = gb_lincomb(ctx, x->n, k1, k2, x->d + start[0], x->ld, ctx->coef, k1, 1.0, 0.0, y->d + start[1], y->ld, 0);
    if (st) return st;
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));   // pinned staging is reused by the next call
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_MultiVecInnerProd(const gcge_gpu_mv *V, const gcge_gpu_mv *W, double *a, const char *is_sym,
                                          const int *start, const int *end, int lda)
{
    if (!V || !W || !a || !start || !end || !is_sym) return GCGE_GPU_ERR_ARG;
    gcge_gpu_ctx *ctx = V->ctx;
    const int k1 = end[0] - start[0], k2 = end[1] - start[1];
    const int sym = strcmp(is_sym, "sym") == 0;
    if (!range_ok(V, start[0], k1) || !range_ok(W, start[1], k2) || V->n != W->n || (sym && k1 != k2) ||
        (k1 > 0 && lda < k1))
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (k1 <= 0 || k2 <= 0) return GCGE_GPU_OK;
    int st = gb_coef(ctx, (size_t)k1 * k2 + 1);
    if (!st) st = gb_pinned(ctx, (size_t)k1 * k2 + 1);
    if (st) return st;
    st = gb_gram(ctx, V->n, k1, k2, V->d + start[0], V->ld, W->d + start[1], W->ld, ctx->coef, k1, sym);
    if (st) return st;
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->pinned, ctx->coef, sizeof(double) * (size_t)k1 * k2, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    for (int j = 0; j < k2; ++j) memcpy(a + (size_t)j * lda, ctx->pinned + (size_t)j * k1, sizeof(double) * k1);
    return GCGE_GPU_OK;
}

__global__ void k_swap_cols(int n, int k, double *A, long lda, double *B, long ldb)
{
    const long total = (long)n * k;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
        const long r = t / k;
        const int c = (int)(t - r * k);
        const double a = A[r * lda + c];
        A[r * lda + c] = B[r * ldb + c];
        B[r * ldb + c] = a;
    }
}

extern "C" int GCGE_GPU_MultiVecSwap(gcge_gpu_mv *V1, gcge_gpu_mv *V2, const int *start, const int *end)
{
    if (!V1 || !V2 || !start || !end) return GCGE_GPU_ERR_ARG;
    gcge_gpu_ctx *ctx = V1->ctx;
    const int k = end[0] - start[0];
    if (k != end[1] - start[1] || !range_ok(V1, start[0], k) || !range_ok(V2, start[1], k) || V1->n != V2->n)
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (k <= 0) return GCGE_GPU_OK;
    if (V1->d == V2->d && !(start[0] + k <= start[1] || start[1] + k <= start[0])) {
        if (start[0] == start[1]) return GCGE_GPU_OK;
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    }
    long total = (long)V1->n * k;
    long g = (total + 255) / 256, cap = (long)ctx->num_sms * 16;
    GB_LAUNCH(ctx, k_swap_cols, (int)(g < cap ? (g > 0 ? g : 1) : cap), 256, 0, V1->n, k, V1->d + start[0], V1->ld,
              V2->d + start[1], V2->ld);
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_BCG(const gcge_gpu_mat *A, gcge_gpu_mv *RHS, int r_start, gcge_gpu_mv *W, int w_start, int k,
                            int cg_max_it, double cg_rate, int precision)
{
    if (!A || !RHS || !W) return GCGE_GPU_ERR_ARG;
    gcge_gpu_ctx *ctx = A->ctx;
    if (!range_ok(RHS, r_start, k) || !range_ok(W, w_start, k) || RHS->n != A->n || W->n != A->n ||
        (precision && !A->v32))
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (k <= 0) return GCGE_GPU_OK;
    size_t bytes = gb_bcg_work_bytes(A->n, k, precision);
    void *work = nullptr;
    CUDA_TRY(ctx, cudaMalloc(&work, bytes));
    gb_bcg_args args;
    memset(&args, 0, sizeof(args));
    args.n = A->n;
    args.k = k;
    args.max_it = cg_max_it;
    args.precision = precision;
    args.rate = cg_rate;
    int st = gb_bcg(ctx, A, RHS->d + r_start, RHS->ld, W->d + w_start, W->ld, &args, work, bytes);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(work);
    return st;
}

// ---------------------------------------------------------------- orthonormalisation
extern "C" int gb_orth_ws_alloc(gcge_gpu_ctx *ctx, gb_orth_ws *ws, int n, int max_width, int max_start)
{
    memset(ws, 0, sizeof(*ws));
    ws->ctx = ctx;
    ws->max_width = max_width;
    ws->max_start = max_start;
    ws->ld1 = (max_width + 1) & ~1;
    size_t kk = (size_t)max_width * max_width;
    // Gram blocks up to [V W]^T (B W): (max_start + max_width) x max_width
    size_t sk = ((size_t)(max_start > 0 ? max_start : 1) + max_width) * max_width;
    ws->g_cap = kk > sk ? kk : sk;
    if (gb_dev_alloc(ctx, (void **)&ws->T1, sizeof(double) * (size_t)n * ws->ld1) != GCGE_GPU_OK ||
        gb_dev_alloc(ctx, (void **)&ws->G, sizeof(double) * (kk > sk ? kk : sk)) != GCGE_GPU_OK ||
        gb_dev_alloc(ctx, (void **)&ws->Tm, sizeof(double) * kk) != GCGE_GPU_OK ||
        gb_dev_alloc(ctx, (void **)&ws->Cm, sizeof(double) * ((size_t)max_start + max_width) * max_width) != GCGE_GPU_OK ||
        gb_dev_alloc(ctx, (void **)&ws->chol_work, sizeof(double) * 2 * kk) != GCGE_GPU_OK ||
        gb_dev_alloc(ctx, (void **)&ws->small, sizeof(double) * 64) != GCGE_GPU_OK ||
        gb_dev_alloc(ctx, (void **)&ws->kept_dev, sizeof(int) * 4) != GCGE_GPU_OK ||
        gb_dev_alloc(ctx, (void **)&ws->ev_work, sizeof(double) * gb_syevx_work_doubles(max_width)) != GCGE_GPU_OK ||
        gb_dev_alloc(ctx, (void **)&ws->ev_val, sizeof(double) * max_width) != GCGE_GPU_OK ||
        gb_dev_alloc(ctx, (void **)&ws->ev_info, sizeof(int) * 4) != GCGE_GPU_OK) {
        gb_orth_ws_free(ws);
        return gb_fail(ctx, GCGE_GPU_ERR_NOMEM);
    }
    return GCGE_GPU_OK;
}

extern "C" void gb_orth_ws_free(gb_orth_ws *ws)
{
    gb_dev_free(ws->ctx, ws->T1);
    gb_dev_free(ws->ctx, ws->G);
    gb_dev_free(ws->ctx, ws->Tm);
    gb_dev_free(ws->ctx, ws->Cm);
    gb_dev_free(ws->ctx, ws->chol_work);
    gb_dev_free(ws->ctx, ws->small);
    gb_dev_free(ws->ctx, ws->kept_dev);
    gb_dev_free(ws->ctx, ws->ev_work);
    gb_dev_free(ws->ctx, ws->ev_val);
    gb_dev_free(ws->ctx, ws->ev_info);
    memset(ws, 0, sizeof(*ws));
}

// Cholesky-QR of W (k columns) in the B inner product, with deflation: passes
// first .. 1 of the two (relative deflation tolerance 1e-12, then 1e-14).
static int cholqr2(gcge_gpu_ctx *ctx, int n, double *W, long ldw, int *k_io, const gcge_gpu_mat *B, double zero_tol,
                   gb_orth_ws *ws, int first = 0)
{
    int k = *k_io;
    for (int pass = first; pass < 2 && k > 0; ++pass) {
        const double *BW = W;
        long ldbw = ldw;
        int st;
        if (B) {
            if ((st = gb_spmm(ctx, B, W, ldw, ws->T1, ws->ld1, k, 1.0, nullptr, 0.0, nullptr))) return st;
            BW = ws->T1;
            ldbw = ws->ld1;
        }
        if ((st = gb_gram(ctx, n, k, k, W, ldw, BW, ldbw, ws->G, k, 1))) return st;
        const double rel = pass == 0 ? 1e-12 : 1e-14;
        if ((st = gb_chol_deflate(ctx, k, ws->G, k, ws->Tm, ws->kept_dev, zero_tol, rel, ws->chol_work))) return st;
        int kept = 0;
        CUDA_TRY(ctx, cudaMemcpyAsync(&kept, ws->kept_dev, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (kept <= 0) {
            *k_io = 0;
            return GCGE_GPU_OK;
        }
        if (gb_lincomb_inplace_ok(ctx, k, kept)) {
            if ((st = gb_lincomb(ctx, n, k, kept, W, ldw, ws->Tm, k, 1.0, 0.0, W, ldw, kept == k))) return st;
        } else {
            if ((st = gb_lincomb(ctx, n, k, kept, W, ldw, ws->Tm, k, 1.0, 0.0, ws->T1, ws->ld1, kept == k))) return st;
            if ((st = gb_axpby(ctx, n, kept, 1.0, ws->T1, ws->ld1, 0.0, W, ldw))) return st;
        }
        k = kept;
    }
    *k_io = k;
    return GCGE_GPU_OK;
}

// The first projection pass is W -= V (V^T B W). The second computes B W once
// more and, in the same Gram call, both G2 = V^T B W and W^T B W (V and W are
// contiguous columns of one block). When no third pass is needed, the first
// Cholesky-QR Gram of W - V G2 follows without another B product:
//   (W - V G2)^T B (W - V G2) = W^T B W - G2^T G2,   as V^T B V = I,
// and the projection and R^-1 are applied together: W <- [V W] [[-G2 T], [T]].
// The second Cholesky-QR pass forms its B product afresh (it exists to repair
// the rounding of the first).
extern "C" int gb_orthonormalize(gcge_gpu_ctx *ctx, int n, double *V, long ldv, int start, int *end,
                                 const gcge_gpu_mat *B, int max_reorth_time, double zero_tol, gb_orth_ws *ws)
{
    int k = *end - start;
    if (k <= 0) return GCGE_GPU_OK;
    if (k > ws->max_width || start > ws->max_start || ((size_t)start + k) * k > ws->g_cap)
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    double *W = V + start;
    int st;
    auto bprod = [&](const double **BW, long *ldbw) -> int {
        *BW = W;
        *ldbw = ldv;
        if (!B) return GCGE_GPU_OK;
        *BW = ws->T1;
        *ldbw = ws->ld1;
        return gb_spmm(ctx, B, W, ldv, ws->T1, ws->ld1, k, 1.0, nullptr, 0.0, nullptr);
    };
    if (start > 0) {
        const int passes = max_reorth_time < 1 ? 1 : max_reorth_time;
        const double *BW;
        long ldbw;
        // projection pass 1
        if ((st = bprod(&BW, &ldbw))) return st;
        if ((st = gb_gram(ctx, n, start, k, V, ldv, BW, ldbw, ws->G, start, 0))) return st;
        if ((st = gb_lincomb(ctx, n, start, k, V, ldv, ws->G, start, -1.0, 1.0, W, ldv, 0))) return st;
        if (passes == 1) {
            if ((st = cholqr2(ctx, n, W, ldv, &k, B, zero_tol, ws))) return st;
            *end = start + k;
            return GCGE_GPU_OK;
        }
        if (passes > 2 && (st = gb_frobenius(ctx, start, k, ws->G, start, ws->small))) return st;
        // projection pass 2: [V W]^T B W in one Gram (ld start + k)
        const int ldg = start + k;
        if ((st = bprod(&BW, &ldbw))) return st;
        if ((st = gb_gram(ctx, n, ldg, k, V, ldv, BW, ldbw, ws->G, ldg, 0))) return st;
        bool third = false;
        if (passes > 2) {
            // "twice is enough": a third pass only if the second still removed a sizeable part
            if ((st = gb_frobenius(ctx, start, k, ws->G, ldg, ws->small + 1))) return st;
            double h[2];
            CUDA_TRY(ctx, cudaMemcpyAsync(h, ws->small, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
            CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
            third = h[1] > 1e-10 * h[0];
        }
        if (third) {
            if ((st = gb_lincomb(ctx, n, start, k, V, ldv, ws->G, ldg, -1.0, 1.0, W, ldv, 0))) return st;
            for (int pass = 2; pass < passes; ++pass) {
                if ((st = bprod(&BW, &ldbw))) return st;
                if ((st = gb_gram(ctx, n, start, k, V, ldv, BW, ldbw, ws->G, start, 0))) return st;
                if ((st = gb_lincomb(ctx, n, start, k, V, ldv, ws->G, start, -1.0, 1.0, W, ldv, 0))) return st;
            }
            if ((st = cholqr2(ctx, n, W, ldv, &k, B, zero_tol, ws))) return st;
            *end = start + k;
            return GCGE_GPU_OK;
        }
        // first Cholesky-QR on S = W^T B W - G2^T G2, recombination in one linear combination
        double *S = ws->G + start;
        if ((st = gb_small_gemm(ctx, 'T', 'N', k, k, start, -1.0, ws->G, ldg, ws->G, ldg, 1.0, S, ldg))) return st;
        if ((st = gb_chol_deflate(ctx, k, S, ldg, ws->Tm, ws->kept_dev, zero_tol, 1e-12, ws->chol_work))) return st;
        int kept = 0;
        CUDA_TRY(ctx, cudaMemcpyAsync(&kept, ws->kept_dev, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (kept <= 0) {
            *end = start;
            return GCGE_GPU_OK;
        }
        if ((st = gb_small_gemm(ctx, 'N', 'N', start, kept, k, -1.0, ws->G, ldg, ws->Tm, k, 0.0, ws->Cm, ldg)))
            return st;
        CUDA_TRY(ctx, cudaMemcpy2DAsync(ws->Cm + start, sizeof(double) * ldg, ws->Tm, sizeof(double) * k,
                                        sizeof(double) * k, kept, cudaMemcpyDeviceToDevice, ctx->stream));
        if (gb_lincomb_inplace_ok(ctx, ldg, kept)) {
            if ((st = gb_lincomb(ctx, n, ldg, kept, V, ldv, ws->Cm, ldg, 1.0, 0.0, W, ldv, 0))) return st;
        } else {
            if ((st = gb_lincomb(ctx, n, ldg, kept, V, ldv, ws->Cm, ldg, 1.0, 0.0, ws->T1, ws->ld1, 0))) return st;
            if ((st = gb_axpby(ctx, n, kept, 1.0, ws->T1, ws->ld1, 0.0, W, ldv))) return st;
        }
        k = kept;
        if ((st = cholqr2(ctx, n, W, ldv, &k, B, zero_tol, ws, 1))) return st;
        *end = start + k;
        return GCGE_GPU_OK;
    }
    if ((st = cholqr2(ctx, n, W, ldv, &k, B, zero_tol, ws))) return st;
    *end = start + k;
    return GCGE_GPU_OK;
}

// ---------------------------------------------------------------- orthonormalisation variants
extern "C" int gb_orth_kind(const char *t)
{
    if (!t || !t[0] || strcmp(t, "multi") == 0) return GB_ORTH_MULTI;
    if (strcmp(t, "cbgs") == 0) return GB_ORTH_CBGS;
    if (strcmp(t, "scbgs") == 0) return GB_ORTH_SCBGS;
    return GB_ORTH_GS;                                   // "bgs" and the reference's fallback branch
}

// T[:, 0:kept) = Q[:, f:k) diag(theta[f:k])^-1/2 with f one past the last
// eigenvalue below the tolerance (ascending theta; the reference's
// tmp_eval_nonzero_start), kept = k - f; one block. A direction is kept when
// its norm sqrt(theta) exceeds the zero tolerance and theta exceeds 1e-12 of the
// largest eigenvalue -- the two tests of the Cholesky-QR form on its pivots (the
// eigensolver resolves theta only to ~1e-16 theta_max)
__global__ void k_eig_inv_sqrt(int k, const double *__restrict__ Q, int ldq, const double *__restrict__ theta,
                               double tol, double *__restrict__ T, int ldt, int *__restrict__ kept)
{
    __shared__ int f;
    if (threadIdx.x == 0) {
        const double rel = theta[k - 1] > 0.0 ? 1e-12 * theta[k - 1] : 0.0;
        int s = 0;
        for (int j = 0; j < k; ++j)
            if (!(theta[j] > tol * tol && theta[j] > rel)) s = j + 1;
        f = s;
        *kept = k - s;
    }
    __syncthreads();
    const int kp = k - f;
    for (int e = threadIdx.x; e < k * kp; e += blockDim.x) {
        const int i = e % k, c = e / k;
        T[i + (long)c * ldt] = Q[i + (long)(c + f) * ldq] / sqrt(theta[c + f]);
    }
}

// one eigenvalue step of W (k columns): W <- W Q theta^-1/2; *k shrinks by the dropped columns
static int eig_orth(gcge_gpu_ctx *ctx, int n, double *W, long ldw, int *k_io, const gcge_gpu_mat *B, double zero_tol,
                    gb_orth_ws *ws)
{
    const int k = *k_io;
    const double *BW = W;
    long ldbw = ldw;
    int st;
    if (B) {
        if ((st = gb_spmm(ctx, B, W, ldw, ws->T1, ws->ld1, k, 1.0, nullptr, 0.0, nullptr))) return st;
        BW = ws->T1;
        ldbw = ws->ld1;
    }
    if ((st = gb_gram(ctx, n, k, k, W, ldw, BW, ldbw, ws->G, k, 1))) return st;
    if ((st = gb_syevx(ctx, k, ws->G, k, 1, k, ws->ev_val, ws->Tm, k, ws->ev_work, ws->ev_info))) return st;
    GB_LAUNCH(ctx, k_eig_inv_sqrt, 1, 256, 0, k, ws->Tm, k, ws->ev_val, zero_tol, ws->Cm, k, ws->kept_dev);
    int h[2] = {0, 0};
    CUDA_TRY(ctx, cudaMemcpyAsync(h, ws->kept_dev, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaMemcpyAsync(h + 1, ws->ev_info, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (h[1]) return gb_fail(ctx, GCGE_GPU_ERR_EIGSOLVE);
    const int kept = h[0];
    if (kept <= 0) {
        *k_io = 0;
        return GCGE_GPU_OK;
    }
    if (gb_lincomb_inplace_ok(ctx, k, kept)) {
        if ((st = gb_lincomb(ctx, n, k, kept, W, ldw, ws->Cm, k, 1.0, 0.0, W, ldw, 0))) return st;
    } else {
        if ((st = gb_lincomb(ctx, n, k, kept, W, ldw, ws->Cm, k, 1.0, 0.0, ws->T1, ws->ld1, 0))) return st;
        if ((st = gb_axpby(ctx, n, kept, 1.0, ws->T1, ws->ld1, 0.0, W, ldw))) return st;
    }
    *k_io = kept;
    return GCGE_GPU_OK;
}

// block projection W -= V (V^T B W), V = the first `start` columns
static int block_project(gcge_gpu_ctx *ctx, int n, double *V, long ldv, int start, int k, const gcge_gpu_mat *B,
                         gb_orth_ws *ws)
{
    double *W = V + start;
    const double *BW = W;
    long ldbw = ldv;
    int st;
    if (B) {
        if ((st = gb_spmm(ctx, B, W, ldv, ws->T1, ws->ld1, k, 1.0, nullptr, 0.0, nullptr))) return st;
        BW = ws->T1;
        ldbw = ws->ld1;
    }
    if ((st = gb_gram(ctx, n, start, k, V, ldv, BW, ldbw, ws->G, start, 0))) return st;
    return gb_lincomb(ctx, n, start, k, V, ldv, ws->G, start, -1.0, 1.0, W, ldv, 0);
}

// column-by-column Gram-Schmidt in the B inner product, two projections per
// column; a column whose B-norm falls to the zero tolerance, or whose squared
// B-norm to 1e-24 of its value before the projections, is replaced by the last one
static int gs_orth(gcge_gpu_ctx *ctx, int n, double *V, long ldv, int start, int *end, const gcge_gpu_mat *B,
                   double zero_tol, gb_orth_ws *ws)
{
    int k = *end - start, st;
    auto bnorm2 = [&](int col, double *out) -> int {
        const double *bw = V + col;
        long ld = ldv;
        int s;
        if (B) {
            if ((s = gb_spmm(ctx, B, V + col, ldv, ws->T1, ws->ld1, 1, 1.0, nullptr, 0.0, nullptr))) return s;
            bw = ws->T1;
            ld = ws->ld1;
        }
        if ((s = gb_gram(ctx, n, 1, 1, V + col, ldv, bw, ld, ws->small, 1, 0))) return s;
        CUDA_TRY(ctx, cudaMemcpyAsync(out, ws->small, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        return GCGE_GPU_OK;
    };
    for (int j = 0; j < k;) {
        const int col = start + j;
        double before = 0.0, after = 0.0;
        if ((st = bnorm2(col, &before))) return st;
        for (int pass = 0; pass < 2 && col > 0; ++pass) {
            const double *bw = V + col;
            long ld = ldv;
            if (B) {
                if ((st = gb_spmm(ctx, B, V + col, ldv, ws->T1, ws->ld1, 1, 1.0, nullptr, 0.0, nullptr))) return st;
                bw = ws->T1;
                ld = ws->ld1;
            }
            if ((st = gb_gram(ctx, n, col, 1, V, ldv, bw, ld, ws->G, col, 0))) return st;
            if ((st = gb_lincomb(ctx, n, col, 1, V, ldv, ws->G, col, -1.0, 1.0, V + col, ldv, 0))) return st;
        }
        if ((st = bnorm2(col, &after))) return st;
        if (!(sqrt(after) > zero_tol) || !(after > 1e-24 * before)) {
            // dependent column: the last unprocessed column takes its place
            if (j != k - 1 && (st = gb_axpby(ctx, n, 1, 1.0, V + start + k - 1, ldv, 0.0, V + col, ldv))) return st;
            --k;
            continue;
        }
        if ((st = gb_axpby(ctx, n, 1, 1.0 / sqrt(after), V + col, ldv, 0.0, V + col, ldv))) return st;
        ++j;
    }
    *end = start + k;
    return GCGE_GPU_OK;
}

extern "C" int gb_orthonormalize_kind(gcge_gpu_ctx *ctx, int n, double *V, long ldv, int start, int *end,
                                      const gcge_gpu_mat *B, int max_reorth_time, double zero_tol, gb_orth_ws *ws,
                                      int kind)
{
    if (kind == GB_ORTH_MULTI) return gb_orthonormalize(ctx, n, V, ldv, start, end, B, max_reorth_time, zero_tol, ws);
    int k = *end - start;
    if (k <= 0) return GCGE_GPU_OK;
    if (k > ws->max_width || start > ws->max_start || ((size_t)start + k) * k > ws->g_cap)
        return gb_fail(ctx, GCGE_GPU_ERR_ARG);
    if (kind == GB_ORTH_GS) return gs_orth(ctx, n, V, ldv, start, end, B, zero_tol, ws);
    int st;
    if (start > 0)
        for (int pass = 0; pass < 2; ++pass)
            if ((st = block_project(ctx, n, V, ldv, start, k, B, ws))) return st;
    const int rounds = kind == GB_ORTH_SCBGS ? 2 : 1;
    for (int r = 0; r < rounds && k > 0; ++r)
        if ((st = eig_orth(ctx, n, V + start, ldv, &k, B, zero_tol, ws))) return st;
    *end = start + k;
    return GCGE_GPU_OK;
}

extern "C" int GCGE_GPU_OrthonormalizeType(gcge_gpu_mv *W, int start, int *end, const gcge_gpu_mat *B,
                                           int max_reorth_time, double orth_zero_tol, const char *w_orth_type)
{
    if (!W || !end || start < 0 || *end < start || *end > W->ncols || (B && B->n != W->n))
        return gb_fail(W ? W->ctx : nullptr, GCGE_GPU_ERR_ARG);
    gcge_gpu_ctx *ctx = W->ctx;
    gb_orth_ws ws;
    int st = gb_orth_ws_alloc(ctx, &ws, W->n, *end - start > 0 ? *end - start : 1, start);
    if (st) return st;
    st = gb_orthonormalize_kind(ctx, W->n, W->d, W->ld, start, end, B, max_reorth_time, orth_zero_tol + DBL_EPSILON,
                                &ws, gb_orth_kind(w_orth_type));
    cudaStreamSynchronize(ctx->stream);
    gb_orth_ws_free(&ws);
    return st;
}

extern "C" int GCGE_GPU_Orthonormalize(gcge_gpu_mv *W, int start, int *end, const gcge_gpu_mat *B, int max_reorth_time,
                                       double orth_zero_tol)
{
    if (!W || !end || start < 0 || *end < start || *end > W->ncols || (B && B->n != W->n))
        return gb_fail(W ? W->ctx : nullptr, GCGE_GPU_ERR_ARG);
    gcge_gpu_ctx *ctx = W->ctx;
    gb_orth_ws ws;
    int st = gb_orth_ws_alloc(ctx, &ws, W->n, *end - start > 0 ? *end - start : 1, start);
    if (st) return st;
    st = gb_orthonormalize(ctx, W->n, W->d, W->ld, start, end, B, max_reorth_time, orth_zero_tol + DBL_EPSILON, &ws);
    cudaStreamSynchronize(ctx->stream);
    gb_orth_ws_free(&ws);
    return st;
}
