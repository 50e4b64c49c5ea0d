/* gb_csrio.c -- CSR matrices from files, on the host.
 *
 * Text: the reference's format (CSR_ReadMatFile, app/csr/gcge_app_csr.c:185-236):
 * nrow, ncol, nnz, then RowPtr[nrow + 1], KCol[nnz], Entries[nnz], separated by
 * white space, indices from 0. The reference reads it with fscanf and exits on
 * a missing file; here every failure is a status code and the arrays are
 * checked (monotone row pointers from 0 to nnz, columns in range).
 *
 * Binary: the same arrays behind a 24-byte header, little endian:
 *   "GCGECSR" 0x01 | int32 nrow | int32 ncol | int64 nnz |
 *   int32 RowPtr[nrow + 1] | int32 KCol[nnz] | float64 Entries[nnz]
 * (no counterpart in the reference; a fixed-size record that loads with three
 * reads instead of a text parse).
 *
 * GCGE_GPU_MatCreateFromFile picks the form by the header and uploads the matrix
 * (the role of GCGE_CSR_Solver_Init's reading and setup, app/csr/gcge_app_csr.c:92-124).
 */
#include <errno.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gcge_gb300.h"

static const char CSR_MAGIC[8] = {'G', 'C', 'G', 'E', 'C', 'S', 'R', 1};

static int little_endian(void)
{
    const uint16_t one = 1;
    unsigned char b;
    memcpy(&b, &one, 1);
    return b == 1;
}

/* row pointers from 0 to nnz, non-decreasing; columns in [0, ncol) */
static int check_arrays(int nrow, int ncol, long long nnz, const int *rp, const int *ci)
{
    if (rp[0] != 0 || rp[nrow] != nnz) return GCGE_GPU_ERR_CSR;
    for (int i = 0; i < nrow; ++i)
        if (rp[i + 1] < rp[i]) return GCGE_GPU_ERR_CSR;
    for (long long e = 0; e < nnz; ++e)
        if (ci[e] < 0 || ci[e] >= ncol) return GCGE_GPU_ERR_CSR;
    return GCGE_GPU_OK;
}

static int alloc_arrays(int nrow, long long nnz, int **rp, int **ci, double **v)
{
    const size_t nz = nnz > 0 ? (size_t)nnz : 1;
    *rp = (int *)malloc(sizeof(int) * ((size_t)nrow + 1));
    *ci = (int *)malloc(sizeof(int) * nz);
    *v = (double *)malloc(sizeof(double) * nz);
    if (!*rp || !*ci || !*v) {
        free(*rp);
        free(*ci);
        free(*v);
        *rp = NULL;
        *ci = NULL;
        *v = NULL;
        return GCGE_GPU_ERR_NOMEM;
    }
    return GCGE_GPU_OK;
}

void GCGE_GPU_CSRFree(int *rowptr, int *col, double *val)
{
    free(rowptr);
    free(col);
    free(val);
}

/* the whole file in one NUL-terminated buffer */
static char *slurp(const char *path, size_t *len)
{
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    char *buf = NULL;
    size_t cap = 0, n = 0;
    for (;;) {
        if (n + 65536 + 1 > cap) {
            const size_t nc = cap ? 2 * cap : 1 << 20;
            char *nb = (char *)realloc(buf, nc);
            if (!nb) {
                free(buf);
                fclose(f);
                return NULL;
            }
            buf = nb;
            cap = nc;
        }
        const size_t r = fread(buf + n, 1, cap - n - 1, f);
        n += r;
        if (r == 0) break;
    }
    const int err = ferror(f);
    fclose(f);
    if (err) {
        free(buf);
        return NULL;
    }
    buf[n] = '\0';
    *len = n;
    return buf;
}

static int next_long(char **p, long long *out)
{
    char *end;
    errno = 0;
    const long long x = strtoll(*p, &end, 10);
    if (end == *p || errno) return 0;
    *p = end;
    *out = x;
    return 1;
}

static int next_double(char **p, double *out)
{
    char *end;
    const double x = strtod(*p, &end);
    if (end == *p) return 0;
    *p = end;
    *out = x;
    return 1;
}

int GCGE_GPU_CSRReadText(const char *path, int *nrow, int *ncol, int *nnz, int **rowptr, int **col, double **val)
{
    if (!path || !nrow || !ncol || !nnz || !rowptr || !col || !val) return GCGE_GPU_ERR_ARG;
    *rowptr = NULL;
    *col = NULL;
    *val = NULL;
    size_t len = 0;
    char *buf = slurp(path, &len);
    if (!buf) return GCGE_GPU_ERR_IO;
    char *p = buf;
    long long nr, nc, nz;
    int st = GCGE_GPU_ERR_IO;
    if (!next_long(&p, &nr) || !next_long(&p, &nc) || !next_long(&p, &nz)) goto done;
    if (nr <= 0 || nc <= 0 || nz < 0 || nr > 0x7ffffffeLL || nc > 0x7fffffffLL || nz > 0x7fffffffLL) {
        st = GCGE_GPU_ERR_CSR;
        goto done;
    }
    if ((st = alloc_arrays((int)nr, nz, rowptr, col, val))) goto done;
    st = GCGE_GPU_ERR_IO;
    for (long long i = 0; i <= nr; ++i) {
        long long x;
        if (!next_long(&p, &x)) goto fail;
        if (x < 0 || x > nz) {
            st = GCGE_GPU_ERR_CSR;
            goto fail;
        }
        (*rowptr)[i] = (int)x;
    }
    for (long long e = 0; e < nz; ++e) {
        long long x;
        if (!next_long(&p, &x)) goto fail;
        if (x < 0 || x >= nc) {
            st = GCGE_GPU_ERR_CSR;
            goto fail;
        }
        (*col)[e] = (int)x;
    }
    for (long long e = 0; e < nz; ++e)
        if (!next_double(&p, *val + e)) goto fail;
    if ((st = check_arrays((int)nr, (int)nc, nz, *rowptr, *col))) goto fail;
    *nrow = (int)nr;
    *ncol = (int)nc;
    *nnz = (int)nz;
    st = GCGE_GPU_OK;
    goto done;
fail:
    GCGE_GPU_CSRFree(*rowptr, *col, *val);
    *rowptr = NULL;
    *col = NULL;
    *val = NULL;
done:
    free(buf);
    return st;
}

int GCGE_GPU_CSRReadBinary(const char *path, int *nrow, int *ncol, int *nnz, int **rowptr, int **col,
                           double **val)
{
    if (!path || !nrow || !ncol || !nnz || !rowptr || !col || !val) return GCGE_GPU_ERR_ARG;
    *rowptr = NULL;
    *col = NULL;
    *val = NULL;
    if (!little_endian()) return GCGE_GPU_ERR_IO;
    FILE *f = fopen(path, "rb");
    if (!f) return GCGE_GPU_ERR_IO;
    char magic[8];
    int32_t nr, nc;
    int64_t nz;
    int st = GCGE_GPU_ERR_IO;
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, CSR_MAGIC, 8) != 0 || fread(&nr, 4, 1, f) != 1 ||
        fread(&nc, 4, 1, f) != 1 || fread(&nz, 8, 1, f) != 1)
        goto done;
    if (nr <= 0 || nc <= 0 || nz < 0 || nr > 0x7ffffffe || nz > 0x7fffffffLL) {
        st = GCGE_GPU_ERR_CSR;
        goto done;
    }
    if ((st = alloc_arrays(nr, nz, rowptr, col, val))) goto done;
    st = GCGE_GPU_ERR_IO;
    if (fread(*rowptr, sizeof(int), (size_t)nr + 1, f) != (size_t)nr + 1 ||
        fread(*col, sizeof(int), (size_t)nz, f) != (size_t)nz || fread(*val, sizeof(double), (size_t)nz, f) != (size_t)nz)
        goto fail;
    if ((st = check_arrays(nr, nc, nz, *rowptr, *col))) goto fail;
    *nrow = nr;
    *ncol = nc;
    *nnz = (int)nz;
    st = GCGE_GPU_OK;
    goto done;
fail:
    GCGE_GPU_CSRFree(*rowptr, *col, *val);
    *rowptr = NULL;
    *col = NULL;
    *val = NULL;
done:
    fclose(f);
    return st;
}

int GCGE_GPU_CSRWriteBinary(const char *path, int nrow, int ncol, int nnz, const int *rowptr, const int *col,
                            const double *val)
{
    if (!path || nrow <= 0 || ncol <= 0 || nnz < 0 || !rowptr || (nnz && (!col || !val))) return GCGE_GPU_ERR_ARG;
    if (!little_endian()) return GCGE_GPU_ERR_IO;
    int st = check_arrays(nrow, ncol, nnz, rowptr, col);
    if (st) return st;
    FILE *f = fopen(path, "wb");
    if (!f) return GCGE_GPU_ERR_IO;
    const int32_t nr = nrow, nc = ncol;
    const int64_t nz = nnz;
    int ok = fwrite(CSR_MAGIC, 1, 8, f) == 8 && fwrite(&nr, 4, 1, f) == 1 && fwrite(&nc, 4, 1, f) == 1 &&
             fwrite(&nz, 8, 1, f) == 1 && fwrite(rowptr, sizeof(int), (size_t)nrow + 1, f) == (size_t)nrow + 1 &&
             fwrite(col, sizeof(int), (size_t)nnz, f) == (size_t)nnz &&
             fwrite(val, sizeof(double), (size_t)nnz, f) == (size_t)nnz;
    if (fclose(f) != 0) ok = 0;
    return ok ? GCGE_GPU_OK : GCGE_GPU_ERR_IO;
}

int GCGE_GPU_MatCreateFromFile(gcge_gpu_ctx *ctx, const char *path, int keep_fp32, gcge_gpu_mat **out)
{
    if (!ctx || !path || !out) return GCGE_GPU_ERR_ARG;
    *out = NULL;
    char magic[8] = {0};
    FILE *f = fopen(path, "rb");
    if (!f) return GCGE_GPU_ERR_IO;
    const size_t got = fread(magic, 1, 8, f);
    fclose(f);
    int nrow = 0, ncol = 0, nnz = 0, *rp = NULL, *ci = NULL;
    double *v = NULL;
    const int st = (got == 8 && memcmp(magic, CSR_MAGIC, 8) == 0)
                       ? GCGE_GPU_CSRReadBinary(path, &nrow, &ncol, &nnz, &rp, &ci, &v)
                       : GCGE_GPU_CSRReadText(path, &nrow, &ncol, &nnz, &rp, &ci, &v);
    if (st) return st;
    int st2 = nrow == ncol ? GCGE_GPU_MatCreate(ctx, nrow, rp, ci, v, keep_fp32, out) : GCGE_GPU_ERR_CSR;
    GCGE_GPU_CSRFree(rp, ci, v);
    return st2;
}
