/*
 * pf_oracle_api.c -- flat handle API over the CPU oracle for ctypes callers.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py through oracle/oracle.py.
 */
#include "pf_oracle.h"

#include <stdlib.h>
#include <string.h>

typedef struct {
    orc_grid g;
    orc_ybus y;
    orc_result r;
    int have_r;
} orc_handle;

void *orc_h_open(const char *path, double v0, double th0, char *err, int errlen) {
    orc_handle *h = (orc_handle *)calloc(1, sizeof(orc_handle));
    if (orc_read_cdf(path, v0, th0, &h->g, err, errlen)) { free(h); return NULL; }
    orc_build_ybus(&h->g, &h->y);
    return h;
}

/* Ybus by calcYbus's rule (metodo = denso) when dense != 0, else calcYbusSp's. */
void orc_h_set_dense_ybus(void *hv, int dense) {
    orc_handle *h = (orc_handle *)hv;
    h->g.dense_ybus = dense != 0;
    orc_ybus_free(&h->y);
    orc_build_ybus(&h->g, &h->y);
}

/* 0: calcYbusSp_eficinte's branch stamps, 1: calcYbusSp_Matpower's (.m input). */
int orc_h_ybus_form(void *hv) { return ((orc_handle *)hv)->g.ybus_form; }
void orc_h_set_ybus_form(void *hv, int form) {
    orc_handle *h = (orc_handle *)hv;
    h->g.ybus_form = form;
    orc_ybus_free(&h->y);
    orc_build_ybus(&h->g, &h->y);
}

void orc_h_close(void *hv) {
    orc_handle *h = (orc_handle *)hv;
    if (!h) return;
    orc_grid_free(&h->g);
    orc_ybus_free(&h->y);
    if (h->have_r) orc_result_free(&h->r);
    free(h);
}

/* dims: nB, nL, nPV, nPQ, slack, nnzY, n_warn, baseMVA(int) */
void orc_h_dims(void *hv, int *d) {
    orc_handle *h = (orc_handle *)hv;
    d[0] = h->g.nB; d[1] = h->g.nL; d[2] = h->g.nPV; d[3] = h->g.nPQ; d[4] = h->g.slack;
    d[5] = h->y.nnz; d[6] = h->g.n_warn; d[7] = (int)h->g.baseMVA;
}

/* bus arrays [nB] each: id, type; V, theta, Pload, Qload, Pg, Qg, gsh, bsh;
 * PV arrays [nPV]: barrasPV, Qmin, Qmax, Vset; PQ [nPQ]: barrasPQ;
 * branch [nL]: de, para, z_re, z_im, bsh_br, tap_re, tap_im, phi */
void orc_h_bus(void *hv, int *id, int *type, double *V, double *th, double *Pl, double *Ql,
               double *Pg, double *Qg, double *gsh, double *bsh) {
    orc_grid *g = &((orc_handle *)hv)->g;
    int n = g->nB;
    memcpy(id, g->id, n * sizeof(int)); memcpy(type, g->type, n * sizeof(int));
    memcpy(V, g->V, n * sizeof(double)); memcpy(th, g->theta, n * sizeof(double));
    memcpy(Pl, g->Pload, n * sizeof(double)); memcpy(Ql, g->Qload, n * sizeof(double));
    memcpy(Pg, g->Pg, n * sizeof(double)); memcpy(Qg, g->Qg, n * sizeof(double));
    memcpy(gsh, g->gsh, n * sizeof(double)); memcpy(bsh, g->bsh, n * sizeof(double));
}
void orc_h_pv(void *hv, int *pv, double *qmin, double *qmax, double *vset, int *pq) {
    orc_grid *g = &((orc_handle *)hv)->g;
    memcpy(pv, g->barrasPV, g->nPV * sizeof(int));
    memcpy(qmin, g->Qmin, g->nPV * sizeof(double));
    memcpy(qmax, g->Qmax, g->nPV * sizeof(double));
    memcpy(vset, g->Vset, g->nPV * sizeof(double));
    memcpy(pq, g->barrasPQ, g->nPQ * sizeof(int));
}
void orc_h_branch(void *hv, int *de, int *pa, double *zr, double *zi, double *b, double *tr,
                  double *ti, double *phi) {
    orc_grid *g = &((orc_handle *)hv)->g;
    int n = g->nL;
    memcpy(de, g->de, n * sizeof(int)); memcpy(pa, g->para, n * sizeof(int));
    memcpy(zr, g->z_re, n * sizeof(double)); memcpy(zi, g->z_im, n * sizeof(double));
    memcpy(b, g->bsh_br, n * sizeof(double)); memcpy(tr, g->tap_re, n * sizeof(double));
    memcpy(ti, g->tap_im, n * sizeof(double)); memcpy(phi, g->phi, n * sizeof(double));
}

/* Replace the bus loads / generation / start (scenario variants); Pliq and Qliq
 * are recomputed as in GPU/sistema.h:546-547. */
void orc_h_set_bus(void *hv, const double *Pl, const double *Ql, const double *Pg,
                   const double *Qg, const double *V, const double *th) {
    orc_handle *h = (orc_handle *)hv;
    orc_grid *g = &h->g;
    int n = g->nB;
    if (Pl) memcpy(g->Pload, Pl, n * sizeof(double));
    if (Ql) memcpy(g->Qload, Ql, n * sizeof(double));
    if (Pg) memcpy(g->Pg, Pg, n * sizeof(double));
    if (Qg) memcpy(g->Qg, Qg, n * sizeof(double));
    if (V) memcpy(g->V, V, n * sizeof(double));
    if (th) memcpy(g->theta, th, n * sizeof(double));
    for (int i = 0; i < n; i++) { g->Pliq[i] = g->Pg[i] - g->Pload[i]; g->Qliq[i] = g->Qg[i] - g->Qload[i]; }
    if (V) for (int i = 0; i < g->nPV; i++) g->Vset[i] = g->V[g->barrasPV[i] - 1];
}

void orc_h_ybus(void *hv, int *rowptr, int *col, double *re, double *im) {
    orc_ybus *y = &((orc_handle *)hv)->y;
    memcpy(rowptr, y->rowptr, (y->n + 1) * sizeof(int));
    memcpy(col, y->col, y->nnz * sizeof(int));
    memcpy(re, y->re, y->nnz * sizeof(double));
    memcpy(im, y->im, y->nnz * sizeof(double));
}

void orc_h_pq(void *hv, const double *V, const double *th, double *P, double *Q) {
    orc_pq(&((orc_handle *)hv)->y, V, th, P, Q);
}

/* Jacobian in the reference order; returns nnz (or -needed when cap is short). */
int orc_h_jacobian(void *hv, const double *V, const double *th, const int *pqlim, int nPQlim,
                   int *rowptr, int *col, double *val, int cap) {
    orc_handle *h = (orc_handle *)hv;
    int n = h->g.nB;
    double *P = (double *)calloc(n, sizeof(double)), *Q = (double *)calloc(n, sizeof(double));
    orc_pq(&h->y, V, th, P, Q);
    int dim, nnz, *rp, *cl;
    double *vl;
    orc_jacobian(&h->g, &h->y, V, th, P, Q, pqlim, nPQlim, &dim, &nnz, &rp, &cl, &vl);
    int ret = nnz;
    if (nnz > cap) ret = -nnz;
    else {
        memcpy(rowptr, rp, (dim + 1) * sizeof(int));
        memcpy(col, cl, nnz * sizeof(int));
        memcpy(val, vl, nnz * sizeof(double));
    }
    free(P); free(Q); free(rp); free(cl); free(vl);
    return ret;
}

int orc_h_sparse_solve(int n, const int *rowptr, const int *col, const double *val,
                       const double *b, double *x) {
    return orc_sparse_solve(n, rowptr, col, val, b, x);
}

/* Solve; info: iterations, converged, status, n_events, nPQlim, n_hist. */
int orc_h_solve(void *hv, double tol, int maxit, int lim, int *info, double *final_mm) {
    orc_handle *h = (orc_handle *)hv;
    if (h->have_r) orc_result_free(&h->r);
    orc_opts o = {1.0, 0.0, tol, maxit, lim};
    int st = orc_solve(&h->g, &o, &h->r);
    h->have_r = 1;
    info[0] = h->r.iterations; info[1] = h->r.converged; info[2] = h->r.status;
    info[3] = h->r.n_events; info[4] = h->r.nPQlim; info[5] = h->r.n_hist;
    *final_mm = h->r.final_mismatch;
    return st;
}

/* Results of the last solve: state [nB], flows [nL], hist [n_hist], events 4 x n_events
 * (iteration, bus, PV position, code), limQ [nPV]. */
void orc_h_result(void *hv, double *V, double *th, double *P, double *Q, double *Pdp,
                  double *Ppd, double *Qdp, double *Qpd, double *hist, int *ev, int *limQ) {
    orc_handle *h = (orc_handle *)hv;
    orc_result *r = &h->r;
    int n = h->g.nB, nl = h->g.nL;
    memcpy(V, r->V, n * sizeof(double)); memcpy(th, r->theta, n * sizeof(double));
    memcpy(P, r->Pcalc, n * sizeof(double)); memcpy(Q, r->Qcalc, n * sizeof(double));
    memcpy(Pdp, r->Pdp, nl * sizeof(double)); memcpy(Ppd, r->Ppd, nl * sizeof(double));
    memcpy(Qdp, r->Qdp, nl * sizeof(double)); memcpy(Qpd, r->Qpd, nl * sizeof(double));
    memcpy(hist, r->hist, r->n_hist * sizeof(double));
    for (int i = 0; i < r->n_events; i++) {
        ev[4 * i] = r->ev_iter[i]; ev[4 * i + 1] = r->ev_bus[i];
        ev[4 * i + 2] = r->ev_pvpos[i]; ev[4 * i + 3] = r->ev_code[i];
    }
    memcpy(limQ, r->limQ, h->g.nPV * sizeof(int));
}
