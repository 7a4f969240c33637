/*
 * ORACLE -- test infrastructure only.  A CPU restatement of the ASETS
 * continuous max-flow ALM solvers (maxflow/asets{BinaryMF,Potts,Ishikawa}
 * {2D,3D}_mex.c), used as the checker for libasetscuda and as the timed CPU
 * baseline.  Nothing in the product links or calls it.
 *
 * Pinned against the compiled reference mex sources (tests/test_oracle.py,
 * bit-exact on seeded inputs) and against the committed golden vectors in
 * tests/golden/ generated from those sources.
 */
#ifndef ASETS_ORACLE_H
#define ASETS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_BINARY = 0, ORACLE_POTTS = 1, ORACLE_ISHIKAWA = 2 };

enum {
    ORACLE_OK = 0,
    ORACLE_ERR_ALPHA = 1, /* "alpha(x) must be positive. Exiting..." */
    ORACLE_ERR_ARG = 2,
    ORACLE_ERR_NOMEM = 3
};

typedef struct oracle_problem {
    int model;      /* ORACLE_BINARY / ORACLE_POTTS / ORACLE_ISHIKAWA */
    int dim;        /* 2 or 3 */
    int ny, nx, nz; /* rows (fastest axis), cols, slices (1 in 2D) */
    int nlab;       /* labels (1 for binary) */
    int max_it;
    float err_bound, cc, steps;
    int erru_double; /* 1: accumulate erriter in double instead of float */
    /* inputs, Matlab column-major, label slowest */
    const float *alpha; /* binary: N; Potts: N*L; Ishikawa: >= N*(L-1) */
    const float *cs;    /* binary only */
    const float *ct;    /* binary: N; Potts/Ishikawa: N*L */
    /* optional warm start (all NULL = the reference's init) */
    const float *u0, *ps0, *pt0;
    /* outputs */
    float *u;   /* binary N; Potts N*L; Ishikawa N*(L-1) */
    float *cvg; /* max_it entries, zero past the break */
    int *it_num;
    /* optional final state (may be NULL) */
    float *ps_out; /* binary/Potts: N */
    float *pt_out; /* binary N; Potts N*L; Ishikawa N*L */
} oracle_problem;

int oracle_solve(const oracle_problem *p);

#ifdef __cplusplus
}
#endif

#endif
