/*
 * ref_entry.c -- flat entry point into the compiled GCGE-1.0 reference (the
 * oracle/_ref build). Test infrastructure only.
 *
 * It mirrors GCGE_CSR_Solver_Init (app/csr/gcge_app_csr.c:92-124) with the
 * parameters set before GCGE_SOLVER_Setup, runs GCGE_SOLVER_Solve, and copies
 * the eigenpairs out. The signature matches gcge_oracle_solve so tests can call
 * the restatement and the reference interchangeably.
 */
#define _POSIX_C_SOURCE 199309L
#include <fcntl.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "gcge.h"
#include "gcge_app_csr.h"
#include "gcge_oracle.h"

int gcge_ref_solve(int n, const int *A_rp, const int *A_ci, const double *A_v,
                   const int *B_rp, const int *B_ci, const double *B_v,
                   const gcge_oracle_params *p, double *eval_out, double *evec_out,
                   gcge_oracle_stats *st)
{
    CSR_MAT A = {n, n, A_rp[n], (int *)A_ci, (int *)A_rp, (double *)A_v};
    CSR_MAT B = {n, n, B_rp ? B_rp[n] : 0, (int *)B_ci, (int *)B_rp, (double *)B_v};
    int saved = -1;
    if (p->print_level == 0) {
        fflush(stdout);
        saved = dup(1);
        int devnull = open("/dev/null", O_WRONLY);
        dup2(devnull, 1);
        close(devnull);
    }
    srand((unsigned)p->seed);
    GCGE_SOLVER *s;
    GCGE_SOLVER_Create(&s);
    s->para->nev = p->nev;
    s->para->block_size = p->block_size;
    s->para->ev_max_it = p->ev_max_it;
    s->para->cg_max_it = p->cg_max_it;
    s->para->ev_tol = p->ev_tol;
    s->para->cg_rate = p->cg_rate;
    s->para->orth_para->max_reorth_time = p->max_reorth_time;
    s->para->orth_para->orth_zero_tol = p->orth_zero_tol;
    s->para->orth_para->reorth_tol = p->reorth_tol;
    s->para->orth_para->scbgs_reorth_tol = p->scbgs_reorth_tol;
    s->para->orth_para->criterion_tol = p->criterion_tol;
    s->para->dirichlet_boundary = p->dirichlet_boundary;
    s->para->given_init_evec = p->given_init_evec;
    static char conv[4];
    strncpy(conv, p->conv_type, 3);
    s->para->conv_type = conv;
    static char otype[4];
    if (p->orth_type[0]) {
        strncpy(otype, p->orth_type, 3);
        s->para->orth_type = otype;
    }
    s->para->opt_rr_eig_partly = p->opt_rr_eig_partly;
    static char worth[8];
    if (p->w_orth_type[0]) {
        strncpy(worth, p->w_orth_type, 7);
        s->para->w_orth_type = worth;
    }
    s->para->print_para = 0;
    s->para->print_result = 0;
    int nev = p->nev;
    double *eval = (double *)calloc(nev, sizeof(double));
    CSR_VEC **evec = (CSR_VEC **)malloc(nev * sizeof(CSR_VEC *));
    for (int i = 0; i < nev; ++i) {
        CSR_VecCreateByMat(evec + i, &A);
        if (p->given_init_evec) memcpy(evec[i]->Entries, evec_out + (size_t)i * n, sizeof(double) * n);
    }
    GCGE_SOLVER_SetMatA(s, &A);
    if (B_rp) GCGE_SOLVER_SetMatB(s, &B);
    GCGE_CSR_SetOps(s->ops);
    GCGE_SOLVER_SetEigenvalues(s, eval);
    GCGE_SOLVER_SetEigenvectors(s, (void **)evec);
    GCGE_SOLVER_Setup(s);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    GCGE_SOLVER_Solve(s);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    memcpy(eval_out, eval, sizeof(double) * nev);
    for (int i = 0; i < nev; ++i) memcpy(evec_out + (size_t)i * n, evec[i]->Entries, sizeof(double) * n);
    if (st) {
        st->num_iter = s->para->num_iter;
        st->num_unlock = s->para->num_unlock;
        st->max_res = s->para->max_res;
        st->min_res = s->para->min_res;
        st->sum_res = s->para->sum_res;
        st->wall_s = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
        st->status = 0;
    }
    GCGE_SOLVER_Free_All(&s);
    if (saved >= 0) {
        fflush(stdout);
        dup2(saved, 1);
        close(saved);
    }
    return 0;
}
