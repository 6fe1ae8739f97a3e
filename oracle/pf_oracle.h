/*
 * pf_oracle.h -- CPU oracle for the Newton-Raphson AC power-flow solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * GPU "esparso" solve path (joaovdd/Experience-of-Using-GPU-in-Power-Flow-
 * Computation, GPU/ tree).  It is used by tests/, by __graft_entry__.smoke() and
 * by bench.py's CPU-baseline leg as the checker.  The product (libgbpf) never
 * links, loads or calls it.
 *
 * Parity pin: the restatement is checked against the reference's own CPU-tree
 * functions (reader, Ybus, PQ, Jacobian pattern and values) replaying the GPU
 * driver's control flow, built from the reference sources by oracle/ref/Makefile
 * into oracle/_ref/; tests/golden/ holds the vectors that harness produced.
 *
 * Every function cites the reference file:line it restates.
 */
#ifndef PF_ORACLE_H
#define PF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Host data model of one grid, mirroring struct sistema / barra / ramo
 * (GPU/sistema.h:24-126).  Bus indices are 1-based in file order, like the
 * reference's barrasPV / barrasPQ / barraVO / de / para. */
typedef struct {
    int nB, nL, nPV, nPQ, slack;      /* slack = barraVO (1-based) */
    double baseMVA;
    int *id, *type;                   /* [nB] CDF bus id, bus type column */
    double *V, *theta;                /* [nB] initial state (flat start + setpoints) */
    double *Pload, *Qload, *Pg, *Qg, *Pliq, *Qliq, *gsh, *bsh, *Vbase; /* [nB] */
    int *barrasPV, *barrasPQ;         /* [nPV], [nPQ] ascending, 1-based */
    double *Qmin, *Qmax, *Vset;       /* [nPV] limQinf, limQsup, VfixadaPV */
    int *de, *para;                   /* [nL] 1-based, after parallel merge */
    double *z_re, *z_im, *bsh_br, *tap_re, *tap_im, *phi; /* [nL] */
    int n_warn;                       /* parallel branches with different taps; PV buses with no generator (.m) */
    int dense_ybus;                   /* 1: calcYbus's rule (metodo = denso) */
    int ybus_form;                    /* 0: calcYbusSp_eficinte, 1: calcYbusSp_Matpower (.m input) */
} orc_grid;

/* Row-major CSR Ybus, sorted columns, explicit diagonal (GPU/sistema.h:705-758). */
typedef struct {
    int n, nnz;
    int *rowptr, *col;
    double *re, *im;
} orc_ybus;

typedef struct {
    double v_inicial, theta_inicial, tol;
    int no_max_iter, lim_inj_reat;
} orc_opts;

/* Limit-switch event codes: the five printf lines of chkLimQ
 * (GPU/limiteInjReat.cuh:12,15,23,26,34). */
enum {
    ORC_EV_PV_TO_PQ_MIN = 1,      /* "PV -> PQ (limite superior)"  (Qg < Qmin) */
    ORC_EV_PQMAX_TO_PQMIN = 2,    /* "PQ (limite inferior) -> PQ (limite superior)" */
    ORC_EV_PV_TO_PQ_MAX = 3,      /* "PV -> PQ (limite inferior)"  (Qg > Qmax) */
    ORC_EV_PQMIN_TO_PQMAX = 4,    /* "PQ (limite superior) -> PQ (limite inferior)" */
    ORC_EV_PQ_TO_PV = 5           /* "PQ -> PV" */
};

typedef struct {
    int status;            /* 0 ok, 2 singular Jacobian */
    int converged;
    int iterations;        /* iterPon.iteracao at return (GPU/newtonRaphson.cuh:283,425) */
    double final_mismatch; /* max|g| of the returned state */
    int n_hist;
    double *hist;          /* max|g| per iteration */
    int n_events, cap_events;
    int *ev_iter, *ev_bus, *ev_pvpos, *ev_code;
    int nPQlim;
    int *limQ;             /* [nPV] final limit flags */
    double *V, *theta, *Pcalc, *Qcalc;            /* [nB] */
    double *Pdp, *Ppd, *Qdp, *Qpd;                /* [nL] branch flows */
} orc_result;

/* Read a .cdf (or .cdfx) file: GPU/arquivo.h:250-295, GPU/sistema.h:386-638.
 * Returns 0 on success, nonzero on error (message in err). */
int orc_read_cdf(const char *path, double v_inicial, double theta_inicial,
                 orc_grid *g, char *err, int errlen);
/* Read a MATPOWER case (.m): GPU/m.h:296-622.  Sets ybus_form = 1. */
int orc_read_m(const char *path, double v_inicial, double theta_inicial,
               orc_grid *g, char *err, int errlen);
void orc_grid_free(orc_grid *g);

int orc_build_ybus(const orc_grid *g, orc_ybus *y);
void orc_ybus_free(orc_ybus *y);

void orc_pq(const orc_ybus *y, const double *V, const double *theta,
            double *P, double *Q);

/* Jacobian in the reference's row/column order for the given PQ list
 * (Jstencil0based GPU/esparso.h:61-178 + SpCalcH/L/M/N GPU/Jacobiano.cuh:252-344).
 * Outputs a CSR with dim = nB-1+nPQlim.  Arrays are malloc'd. */
int orc_jacobian(const orc_grid *g, const orc_ybus *y, const double *V,
                 const double *theta, const double *P, const double *Q,
                 const int *pqlim, int nPQlim,
                 int *dim_out, int *nnz_out, int **rowptr, int **col, double **val);

/* Sparse LU solve of A x = b (A in CSR, n x n).  Returns 0 ok, 2 singular. */
int orc_sparse_solve(int n, const int *rowptr, const int *col, const double *val,
                     const double *b, double *x);

/* Full NR solve with the reference GPU driver's control flow
 * (GPU/newtonRaphson.cuh:171-565). */
int orc_solve(const orc_grid *g, const orc_opts *o, orc_result *r);
/* The same solve, writing the reference's verbose_mode dumps to out (FILE *):
 * printAlLim, the per-iteration banner, injections, mismatch, limit lists,
 * max(g), the H/L/M/J value arrays (or the dense JacobianoN when
 * g->dense_ybus), the state, the step and the updated state, in the order and
 * format of GPU/newtonRaphson.cuh:270-563. */
int orc_solve_verbose(const orc_grid *g, const orc_opts *o, orc_result *r, void *out);
void orc_result_free(orc_result *r);

/* Branch flows P/Q from->to and to->from (GPU/PQcalc.cuh:523-557). */
void orc_flows(const orc_grid *g, const orc_ybus *y, const double *V,
               const double *theta, double *Pdp, double *Ppd, double *Qdp,
               double *Qpd);

#ifdef __cplusplus
}
#endif
#endif
