/*
 * pf_oracle.c -- CPU oracle for the Newton-Raphson AC power-flow solve path.
 *
 * TEST INFRASTRUCTURE ONLY (see pf_oracle.h).  Plain C99 restatement of the
 * reference's GPU "esparso" path; each function cites the reference lines it
 * follows.  Independent of the product: its own reader, its own Ybus, and a
 * left-looking Gilbert-Peierls sparse LU with threshold partial pivoting after a
 * minimum-degree column ordering (the product uses a static-pivot block LU on
 * the GPU, so the two solvers share nothing but the mathematics).
 */
#define _GNU_SOURCE
#include "pf_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define PI_REF 3.14159265358979323846 /* the literal used by GPU/sistema.h:526,585 */

/* ------------------------------------------------------------------------- */
/* small helpers                                                             */
/* ------------------------------------------------------------------------- */

static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s ? s : 1);
    if (!p) { fprintf(stderr, "pf_oracle: out of memory\n"); abort(); }
    return p;
}

/* std::string::substr(pos, len) followed by atoi/atof, as every reader line of
 * GPU/sistema.h:386-638 does.  substr throws when pos > size; that is reported
 * as a read error here (*bad = 1). */
static void field(const char *line, size_t n, size_t pos, size_t len, char *buf, int *bad) {
    if (pos > n) { *bad = 1; buf[0] = 0; return; }
    size_t m = n - pos < len ? n - pos : len;
    memcpy(buf, line + pos, m);
    buf[m] = 0;
}
static int fi(const char *line, size_t n, size_t pos, size_t len, int *bad) {
    char b[64]; field(line, n, pos, len, b, bad); return atoi(b);
}
static double fd(const char *line, size_t n, size_t pos, size_t len, int *bad) {
    char b[64]; field(line, n, pos, len, b, bad); return atof(b);
}

/* Smith's (1962) complex division (a+ib)/(c+id). */
static void cdiv(double a, double b, double c, double d, double *re, double *im) {
    if (fabs(c) >= fabs(d)) {
        double r = d / c, den = c + d * r;
        *re = (a + b * r) / den;
        *im = (b - a * r) / den;
    } else {
        double r = c / d, den = c * r + d;
        *re = (a * r + b) / den;
        *im = (b * r - a) / den;
    }
}

/* ------------------------------------------------------------------------- */
/* CDF / CDFX reader                                                         */
/* ------------------------------------------------------------------------- */

/* Column layout of the two fixed-column formats.  CDF: GPU/sistema.h:486-593;
 * CDFX (5-digit ids, every column one to the right): GPU/arquivo.h:96-203. */
typedef struct {
    int id_p, id_l, type_p, v_p, th_p, pl_p, ql_p, pg_p, qg_p, vb_p, qmax_p, qmin_p, gsh_p, bsh_p;
    int de_p, de_l, pa_p, r_p, x_p, b_p, tap_p, phi_p;
} cdf_cols;
static const cdf_cols COLS_CDF = {0, 4, 24, 27, 33, 40, 49, 59, 67, 76, 90, 98, 106, 114,
                                  0, 4, 4, 19, 29, 40, 76, 83};
static const cdf_cols COLS_CDFX = {0, 5, 25, 28, 34, 41, 50, 60, 68, 77, 91, 99, 107, 115,
                                   0, 5, 6, 21, 31, 42, 78, 85};

typedef struct { char **l; size_t *n; int cnt; } lines_t;

static int read_lines(const char *path, lines_t *L) {
    FILE *f = fopen(path, "rb");
    if (!f) return 1;
    int cap = 1024; L->cnt = 0;
    L->l = (char **)xcalloc(cap, sizeof(char *));
    L->n = (size_t *)xcalloc(cap, sizeof(size_t));
    char *buf = NULL; size_t bcap = 0; ssize_t r;
    while ((r = getline(&buf, &bcap, f)) >= 0) {
        size_t n = (size_t)r;
        if (n && buf[n - 1] == '\n') n--; /* std::getline drops only '\n' */
        if (L->cnt == cap) {
            cap *= 2;
            L->l = (char **)realloc(L->l, cap * sizeof(char *));
            L->n = (size_t *)realloc(L->n, cap * sizeof(size_t));
        }
        L->l[L->cnt] = (char *)xcalloc(n + 1, 1);
        memcpy(L->l[L->cnt], buf, n);
        L->n[L->cnt] = n;
        L->cnt++;
    }
    free(buf);
    fclose(f);
    return 0;
}
static void free_lines(lines_t *L) {
    for (int i = 0; i < L->cnt; i++) free(L->l[i]);
    free(L->l); free(L->n);
}

int orc_read_cdf(const char *path, double v_inicial, double theta_inicial,
                 orc_grid *g, char *err, int errlen) {
    memset(g, 0, sizeof(*g));
    /* extension dispatch, GPU/arquivo.h:251-294 */
    const char *dot = strrchr(path, '.');
    char ext[16] = {0};
    if (dot) { for (int i = 0; i < 15 && dot[1 + i]; i++) ext[i] = (char)tolower((unsigned char)dot[1 + i]); }
    const cdf_cols *C;
    if (!strcmp(ext, "cdf")) C = &COLS_CDF;
    else if (!strcmp(ext, "cdfx")) C = &COLS_CDFX;
    else if (!strcmp(ext, "m")) return orc_read_m(path, v_inicial, theta_inicial, g, err, errlen);
    else { snprintf(err, errlen, "unsupported input extension '%s'", ext); return 1; }

    lines_t L;
    if (read_lines(path, &L)) { snprintf(err, errlen, "cannot open %s", path); return 1; }
    int bad = 0;
    if (L.cnt < 2) { free_lines(&L); snprintf(err, errlen, "truncated file"); return 1; }

    /* lerTamanhos, GPU/sistema.h:386-463: count buses by type, then unique (de,para). */
    int li = 2, nB = 0, nPQ = 0, nPV = 0, nslack = 0;
    int bus_start = 2;
    for (; li < L.cnt; li++) {
        if (strstr(L.l[li], "-999")) break;
        nB++;
        int t = fi(L.l[li], L.n[li], C->type_p, 2, &bad);
        if (t == 0 || t == 1) nPQ++;
        else if (t == 2) nPV++;
        else if (t == 3) nslack++;
        else { free_lines(&L); snprintf(err, errlen, "invalid bus type %d", t); return 1; }
    }
    int bus_end = li;
    if (nslack != 1) { free_lines(&L); snprintf(err, errlen, "expected one slack bus, found %d", nslack); return 1; }
    int br_start = bus_end + 2; /* the "-999" line, then the BRANCH DATA header */
    int br_end = br_start;
    while (br_end < L.cnt && !strstr(L.l[br_end], "-999")) br_end++;
    int nraw = br_end - br_start;
    if (nraw < 0) nraw = 0;

    g->nB = nPQ + nPV + 1; /* GPU/sistema.h:554 */
    g->nPQ = nPQ; g->nPV = nPV;
    int n = g->nB;
    g->id = (int *)xcalloc(n, sizeof(int));
    g->type = (int *)xcalloc(n, sizeof(int));
    g->V = (double *)xcalloc(n, sizeof(double));
    g->theta = (double *)xcalloc(n, sizeof(double));
    g->Pload = (double *)xcalloc(n, sizeof(double));
    g->Qload = (double *)xcalloc(n, sizeof(double));
    g->Pg = (double *)xcalloc(n, sizeof(double));
    g->Qg = (double *)xcalloc(n, sizeof(double));
    g->Pliq = (double *)xcalloc(n, sizeof(double));
    g->Qliq = (double *)xcalloc(n, sizeof(double));
    g->gsh = (double *)xcalloc(n, sizeof(double));
    g->bsh = (double *)xcalloc(n, sizeof(double));
    g->Vbase = (double *)xcalloc(n, sizeof(double));
    g->barrasPV = (int *)xcalloc(nPV, sizeof(int));
    g->barrasPQ = (int *)xcalloc(nPQ, sizeof(int));
    g->Qmin = (double *)xcalloc(nPV, sizeof(double));
    g->Qmax = (double *)xcalloc(nPV, sizeof(double));
    g->Vset = (double *)xcalloc(nPV, sizeof(double));
    /* flat start, initBus GPU/sistema.h:254-259 */
    for (int i = 0; i < n; i++) { g->V[i] = v_inicial; g->theta[i] = theta_inicial; }

    /* readCDF, GPU/sistema.h:474-552 */
    g->baseMVA = (double)fi(L.l[0], L.n[0], 31, 6, &bad);
    double base = g->baseMVA;
    int ipv = 0, ipq = 0;
    for (int k = 0; k < nB; k++) {
        const char *s = L.l[bus_start + k]; size_t sn = L.n[bus_start + k];
        int i = k + 1;
        g->id[k] = fi(s, sn, C->id_p, C->id_l, &bad);
        int t = fi(s, sn, C->type_p, 2, &bad);
        g->type[k] = t;
        if (t == 0 || t == 1) {
            g->barrasPQ[ipq++] = i;
        } else if (t == 2) {
            g->barrasPV[ipv] = i;
            g->V[k] = fd(s, sn, C->v_p, 6, &bad);
            g->Vset[ipv] = g->V[k];
            g->Qmax[ipv] = fd(s, sn, C->qmax_p, 7, &bad) / base;
            g->Qmin[ipv] = fd(s, sn, C->qmin_p, 7, &bad) / base;
            ipv++;
        } else { /* t == 3 */
            g->slack = i;
            g->V[k] = fd(s, sn, C->v_p, 6, &bad);
            g->theta[k] = fd(s, sn, C->th_p, 7, &bad) * PI_REF / 180.;
        }
        g->Pload[k] = fd(s, sn, C->pl_p, 9, &bad) / base;
        g->Qload[k] = fd(s, sn, C->ql_p, 10, &bad) / base;
        g->Pg[k] = fd(s, sn, C->pg_p, 8, &bad) / base;
        g->Qg[k] = fd(s, sn, C->qg_p, 8, &bad) / base;
        g->Vbase[k] = fd(s, sn, C->vb_p, 7, &bad);
        g->bsh[k] = fd(s, sn, C->bsh_p, 8, &bad);
        g->gsh[k] = fd(s, sn, C->gsh_p, 8, &bad);
        g->Pliq[k] = g->Pg[k] - g->Pload[k];
        g->Qliq[k] = g->Qg[k] - g->Qload[k];
    }

    /* branches, GPU/sistema.h:556-629: id2i mapping, merge of repeated (de,para). */
    g->de = (int *)xcalloc(nraw, sizeof(int));
    g->para = (int *)xcalloc(nraw, sizeof(int));
    g->z_re = (double *)xcalloc(nraw, sizeof(double));
    g->z_im = (double *)xcalloc(nraw, sizeof(double));
    g->bsh_br = (double *)xcalloc(nraw, sizeof(double));
    g->tap_re = (double *)xcalloc(nraw, sizeof(double));
    g->tap_im = (double *)xcalloc(nraw, sizeof(double));
    g->phi = (double *)xcalloc(nraw, sizeof(double));
    int nL = 0;
    for (int k = 0; k < nraw; k++) {
        const char *s = L.l[br_start + k]; size_t sn = L.n[br_start + k];
        int idde = fi(s, sn, C->de_p, C->de_l, &bad);
        int idpa = fi(s, sn, C->pa_p, 5, &bad);
        int de = 0, pa = 0;
        for (int b = 0; b < n; b++) { if (g->id[b] == idde) { de = b + 1; break; } } /* id2i :465-472 */
        for (int b = 0; b < n; b++) { if (g->id[b] == idpa) { pa = b + 1; break; } }
        if (!de || !pa) {
            free_lines(&L);
            snprintf(err, errlen, "branch %d-%d names an unknown bus", idde, idpa);
            return 1;
        }
        int dup = -1;
        for (int b = 0; b < nL; b++) if (g->de[b] == de && g->para[b] == pa) { dup = b; break; }
        double r = fd(s, sn, C->r_p, 10, &bad), x = fd(s, sn, C->x_p, 11, &bad);
        double a = fd(s, sn, C->tap_p, 6, &bad);
        double ph = fd(s, sn, C->phi_p, 7, &bad) * PI_REF / 180.;
        double bch = fd(s, sn, C->b_p, 10, &bad);
        double tre, tim;
        if (a != 0.) { tre = a * cos(ph); tim = a * sin(ph); }
        else { tre = cos(ph); tim = sin(ph); }
        if (dup < 0) {
            g->de[nL] = de; g->para[nL] = pa;
            g->z_re[nL] = r; g->z_im[nL] = x;
            g->phi[nL] = ph;
            g->tap_re[nL] = tre; g->tap_im[nL] = tim;
            g->bsh_br[nL] = bch;
            nL++;
        } else {
            /* parallel equivalent, GPU/sistema.h:600-624 */
            if (tre != g->tap_re[dup] || tim != g->tap_im[dup]) g->n_warn++;
            double nr = r * g->z_re[dup] - x * g->z_im[dup]; /* aux * z */
            double ni = r * g->z_im[dup] + x * g->z_re[dup];
            double dr = g->z_re[dup] + r, di = g->z_im[dup] + x; /* z + aux */
            cdiv(nr, ni, dr, di, &g->z_re[dup], &g->z_im[dup]);
            if (bch != 0 || g->bsh_br[dup] != 0) g->bsh_br[dup] = 1 / (bch + g->bsh_br[dup]);
            else g->bsh_br[dup] = 0;
        }
    }
    g->nL = nL;
    free_lines(&L);
    if (bad) { snprintf(err, errlen, "a fixed-width field starts past the end of its line"); return 1; }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* MATPOWER case reader: lerArquivoMatPOWEReficiente GPU/m.h:485-599,        */
/* cleanLine / readMatrix GPU/m.h:445-483, storeMatPOWER GPU/m.h:296-443     */
/* ------------------------------------------------------------------------- */

/* cleanLine (GPU/m.h:445-449): drop a '%' comment, then trailing blanks, one
 * ';' and blanks.  A '\r' counts as a blank here. */
static void m_clean(char *s) {
    char *c = strchr(s, '%');
    if (c) *c = 0;
    size_t n = strlen(s);
    while (n && (s[n - 1] == ' ' || s[n - 1] == '\t' || s[n - 1] == '\r')) n--;
    if (n && s[n - 1] == ';') n--;
    while (n && (s[n - 1] == ' ' || s[n - 1] == '\t' || s[n - 1] == '\r')) n--;
    s[n] = 0;
}

/* Removes the first "mpc.<name>[ \t]*=[ \t]*" (plus '[' when bracket) from s
 * and returns 1, as the regex_search + regex_replace pairs of GPU/m.h:505-536
 * do; 0 when s holds no such text. */
static int m_take(char *s, const char *name, int bracket) {
    char key[32];
    snprintf(key, sizeof key, "mpc.%s", name);
    for (char *p = strstr(s, key); p; p = strstr(p + 1, key)) {
        char *q = p + strlen(key);
        while (*q == ' ' || *q == '\t') q++;
        if (*q != '=') continue;
        q++;
        while (*q == ' ' || *q == '\t') q++;
        if (bracket) { if (*q != '[') continue; q++; }
        memmove(p, q, strlen(q) + 1);
        return 1;
    }
    return 0;
}

typedef struct { int rows, cap; int *ncol; double **v; } mmat_t;

/* One matrix row: tokens split on tabs (tokenize(line, "\t"), GPU/m.h:122-142;
 * blanks split too), each read by strtod like std::stod.  A token with no
 * number in front sets *bad (std::stod would throw). */
static void m_row(mmat_t *m, const char *s, int *bad) {
    double *row = NULL;
    int n = 0, cap = 0;
    const char *p = s;
    for (;;) {
        while (*p == '\t' || *p == ' ' || *p == '\r') p++;
        if (!*p) break;
        char *end;
        double v = strtod(p, &end);
        if (end == p) *bad = 1;
        while (*end && *end != '\t' && *end != ' ' && *end != '\r') end++;
        if (n == cap) { cap = cap ? 2 * cap : 16; row = (double *)realloc(row, cap * sizeof(double)); }
        row[n++] = v;
        p = end;
    }
    if (!n) return;
    if (m->rows == m->cap) {
        m->cap = m->cap ? 2 * m->cap : 64;
        m->ncol = (int *)realloc(m->ncol, m->cap * sizeof(int));
        m->v = (double **)realloc(m->v, m->cap * sizeof(double *));
    }
    m->ncol[m->rows] = n;
    m->v[m->rows++] = row;
}

static void m_free(mmat_t *m) {
    for (int i = 0; i < m->rows; i++) free(m->v[i]);
    free(m->ncol); free(m->v);
    memset(m, 0, sizeof(*m));
}

int orc_read_m(const char *path, double v_inicial, double theta_inicial,
               orc_grid *g, char *err, int errlen) {
    memset(g, 0, sizeof(*g));
    lines_t L;
    if (read_lines(path, &L)) { snprintf(err, errlen, "cannot open %s", path); return 1; }
    mmat_t M[3] = {{0}};
    static const char *NAMES[3] = {"bus", "gen", "branch"};
    double base = 0;
    int have_base = 0, bad = 0;
    for (int li = 0; li < L.cnt; li++) {
        char *s = L.l[li];
        m_clean(s);
        if (!*s) continue;
        for (int k = 0; k < 3; k++) {
            if (!m_take(s, NAMES[k], 1)) continue;
            /* readMatrix (GPU/m.h:451-483): rows up to the line holding ']' */
            for (;;) {
                const int last = strchr(s, ']') != NULL;
                if (last) { char *w = s; for (char *r = s; *r; r++) if (*r != ']') *w++ = *r; *w = 0; }
                m_clean(s);
                if (*s) m_row(&M[k], s, &bad);
                if (last || li + 1 >= L.cnt) break;
                s = L.l[++li];
            }
            break;
        }
        if (m_take(s, "baseMVA", 0)) {
            char *w = s;
            for (char *r = s; *r; r++) if (*r != '"' && *r != '\'') *w++ = *r;
            *w = 0;
            char *end;
            base = strtod(s, &end);
            have_base = end != s;
        }
    }
    free_lines(&L);
    int rc = 1;
    if (bad) { snprintf(err, errlen, "a matrix entry is not a number"); goto out; }
    if (!have_base) { snprintf(err, errlen, "mpc.baseMVA not found"); goto out; }
    /* columns read: bus BUS_I..BASE_KV, gen GEN_BUS..QMIN, branch F_BUS..SHIFT */
    static const int NEED[3] = {10, 5, 10};
    for (int k = 0; k < 3; k++)
        for (int i = 0; i < M[k].rows; i++)
            if (M[k].ncol[i] < NEED[k]) {
                snprintf(err, errlen, "mpc.%s row %d has %d columns, %d needed", NAMES[k], i + 1, M[k].ncol[i], NEED[k]);
                goto out;
            }
    /* lerMatPowerEAlocarMemoria GPU/m.h:603-622: sizes by bus type */
    int nbus = M[0].rows, nPQ = 0, nPV = 0, nsl = 0;
    for (int i = 0; i < nbus; i++) {
        int t = (int)M[0].v[i][1];
        if (t == 1) nPQ++;
        else if (t == 2) nPV++;
        else if (t == 3) nsl++;
        else { snprintf(err, errlen, "ERRO: valor de tipo de barra invalido! (%d)", t); goto out; }
    }
    if (nsl != 1) {
        snprintf(err, errlen, nsl ? "ERRO: mais de uma barrra swing definida!" : "no slack bus (type 3) in the file");
        goto out;
    }
    int n = nPQ + nPV + 1;
    g->nB = n; g->nPQ = nPQ; g->nPV = nPV; g->baseMVA = base;
    g->id = (int *)xcalloc(n, sizeof(int));
    g->type = (int *)xcalloc(n, sizeof(int));
    g->V = (double *)xcalloc(n, sizeof(double));
    g->theta = (double *)xcalloc(n, sizeof(double));
    g->Pload = (double *)xcalloc(n, sizeof(double));
    g->Qload = (double *)xcalloc(n, sizeof(double));
    g->Pg = (double *)xcalloc(n, sizeof(double));
    g->Qg = (double *)xcalloc(n, sizeof(double));
    g->Pliq = (double *)xcalloc(n, sizeof(double));
    g->Qliq = (double *)xcalloc(n, sizeof(double));
    g->gsh = (double *)xcalloc(n, sizeof(double));
    g->bsh = (double *)xcalloc(n, sizeof(double));
    g->Vbase = (double *)xcalloc(n, sizeof(double));
    g->barrasPV = (int *)xcalloc(nPV, sizeof(int));
    g->barrasPQ = (int *)xcalloc(nPQ, sizeof(int));
    g->Qmin = (double *)xcalloc(nPV, sizeof(double));
    g->Qmax = (double *)xcalloc(nPV, sizeof(double));
    g->Vset = (double *)xcalloc(nPV, sizeof(double));
    g->ybus_form = 1; /* calcYbusSp_Matpower, GPU/main.cu:78-81 */
    for (int i = 0; i < n; i++) { g->V[i] = v_inicial; g->theta[i] = theta_inicial; }
    /* storeMatPOWER GPU/m.h:304-384 */
    int ipv = 0, ipq = 0;
    for (int k = 0; k < n; k++) {
        const double *b = M[0].v[k];
        const int t = (int)b[1];
        g->id[k] = (int)b[0];
        int gi = -1;
        if (t == 1) {
            g->type[k] = 0;
            g->barrasPQ[ipq++] = k + 1;
        } else {
            g->type[k] = t;
            g->V[k] = b[7];
            if (t == 3) { g->slack = k + 1; g->theta[k] = b[8] * PI_REF / 180.; }
            for (int j = 0; j < M[1].rows; j++) if ((int)M[1].v[j][0] == g->id[k]) { gi = j; break; }
            if (t == 2) {
                g->barrasPV[ipv] = k + 1;
                g->Vset[ipv] = g->V[k];
                /* a PV bus with no generator keeps zero limits */
                if (gi >= 0) { g->Qmax[ipv] = M[1].v[gi][3] / base; g->Qmin[ipv] = M[1].v[gi][4] / base; }
                else g->n_warn++;
                ipv++;
            }
        }
        g->Pload[k] = b[2] / base;
        g->Qload[k] = b[3] / base;
        g->Pg[k] = gi < 0 ? 0 : M[1].v[gi][1] / base;
        g->Qg[k] = gi < 0 ? 0 : M[1].v[gi][2] / base;
        g->Vbase[k] = b[9];
        g->bsh[k] = b[5] / base;
        g->gsh[k] = b[4] / base;
        g->Pliq[k] = g->Pg[k] - g->Pload[k];
        g->Qliq[k] = g->Qg[k] - g->Qload[k];
    }
    /* branches GPU/m.h:386-407: id2i, no merge of repeated pairs */
    int nL = M[2].rows;
    g->de = (int *)xcalloc(nL, sizeof(int));
    g->para = (int *)xcalloc(nL, sizeof(int));
    g->z_re = (double *)xcalloc(nL, sizeof(double));
    g->z_im = (double *)xcalloc(nL, sizeof(double));
    g->bsh_br = (double *)xcalloc(nL, sizeof(double));
    g->tap_re = (double *)xcalloc(nL, sizeof(double));
    g->tap_im = (double *)xcalloc(nL, sizeof(double));
    g->phi = (double *)xcalloc(nL, sizeof(double));
    for (int i = 0; i < nL; i++) {
        const double *r = M[2].v[i];
        const int idde = (int)r[0], idpa = (int)r[1];
        int de = 0, pa = 0;
        for (int b = 0; b < n; b++) { if (g->id[b] == idde) { de = b + 1; break; } } /* id2i GPU/sistema.h:465-472 */
        for (int b = 0; b < n; b++) { if (g->id[b] == idpa) { pa = b + 1; break; } }
        if (!de || !pa) {
            snprintf(err, errlen, "branch %d-%d names an unknown bus", idde, idpa);
            orc_grid_free(g);
            goto out;
        }
        const double a = r[8], ph = r[9] * PI_REF / 180.;
        g->de[i] = de; g->para[i] = pa;
        g->z_re[i] = r[2]; g->z_im[i] = r[3];
        g->phi[i] = ph;
        if (a != 0.) { g->tap_re[i] = a * cos(ph); g->tap_im[i] = a * sin(ph); }
        else { g->tap_re[i] = cos(ph); g->tap_im[i] = sin(ph); }
        g->bsh_br[i] = r[4];
    }
    g->nL = nL;
    rc = 0;
out:
    for (int k = 0; k < 3; k++) m_free(&M[k]);
    return rc;
}

void orc_grid_free(orc_grid *g) {
    free(g->id); free(g->type); free(g->V); free(g->theta); free(g->Pload); free(g->Qload);
    free(g->Pg); free(g->Qg); free(g->Pliq); free(g->Qliq); free(g->gsh); free(g->bsh);
    free(g->Vbase); free(g->barrasPV); free(g->barrasPQ); free(g->Qmin); free(g->Qmax);
    free(g->Vset); free(g->de); free(g->para); free(g->z_re); free(g->z_im); free(g->bsh_br);
    free(g->tap_re); free(g->tap_im); free(g->phi);
    memset(g, 0, sizeof(*g));
}

/* ------------------------------------------------------------------------- */
/* Ybus                                                                      */
/* ------------------------------------------------------------------------- */

typedef struct { int r, c, ord; double re, im; } trip_t;
static int trip_cmp(const void *a, const void *b) {
    const trip_t *x = (const trip_t *)a, *y = (const trip_t *)b;
    if (x->r != y->r) return x->r < y->r ? -1 : 1;
    if (x->c != y->c) return x->c < y->c ? -1 : 1;
    return x->ord < y->ord ? -1 : (x->ord > y->ord);
}

/* calcYbusSp_eficinte, GPU/sistema.h:705-758.  The triplets are summed per
 * (row, col) in insertion order, which is what Eigen's setFromTriplets does
 * (branch stamps in branch order, then the bus shunts). */
int orc_build_ybus(const orc_grid *g, orc_ybus *y) {
    int n = g->nB, nt = 4 * g->nL + n, k = 0;
    trip_t *t = (trip_t *)xcalloc(nt, sizeof(trip_t));
    for (int i = 0; i < g->nL; i++) {
        double ar, ai; /* aux = 1/z */
        cdiv(1., 0., g->z_re[i], g->z_im[i], &ar, &ai);
        int f = g->de[i] - 1, to = g->para[i] - 1;
        double vr, vi;
        double d = hypot(g->tap_re[i], g->tap_im[i]);
        d = 1. / (d * d);
        if (g->ybus_form == 1 && !g->dense_ybus) {
            /* calcYbusSp_Matpower (GPU/sistema.h:760-855): Yft = (-1/conj(t))/z,
             * Ytf = (-1/t)/z, Yff = (1/z + j b/2)/|t|^2, Ytt = 1/z + j b/2, summed
             * through the incidence products Cf'Yf + Ct'Yt + Ysh */
            double ur, ui;
            cdiv(-1., 0., g->tap_re[i], -g->tap_im[i], &ur, &ui);
            cdiv(ur, ui, g->z_re[i], g->z_im[i], &vr, &vi);
            t[k] = (trip_t){f, to, k, vr, vi}; k++;
            cdiv(-1., 0., g->tap_re[i], g->tap_im[i], &ur, &ui);
            cdiv(ur, ui, g->z_re[i], g->z_im[i], &vr, &vi);
            t[k] = (trip_t){to, f, k, vr, vi}; k++;
            t[k] = (trip_t){f, f, k, ar * d, (ai + g->bsh_br[i] / 2.) * d}; k++;
            t[k] = (trip_t){to, to, k, ar, ai + g->bsh_br[i] / 2.}; k++;
            continue;
        }
        cdiv(-ar, -ai, g->tap_re[i], -g->tap_im[i], &vr, &vi); /* -aux/conj(t) */
        t[k] = (trip_t){f, to, k, vr, vi}; k++;
        cdiv(-ar, -ai, g->tap_re[i], g->tap_im[i], &vr, &vi);  /* -aux/t */
        t[k] = (trip_t){to, f, k, vr, vi}; k++;
        t[k] = (trip_t){f, f, k, d * ar, d * ai + g->bsh_br[i] / 2.}; k++;
        t[k] = (trip_t){to, to, k, ar, ai + g->bsh_br[i] / 2.}; k++;
    }
    for (int i = 0; i < n; i++) { t[k] = (trip_t){i, i, k, g->gsh[i], g->bsh[i]}; k++; }
    qsort(t, nt, sizeof(trip_t), trip_cmp);
    y->n = n;
    y->rowptr = (int *)xcalloc(n + 1, sizeof(int));
    y->col = (int *)xcalloc(nt, sizeof(int));
    y->re = (double *)xcalloc(nt, sizeof(double));
    y->im = (double *)xcalloc(nt, sizeof(double));
    int nnz = 0;
    for (int i = 0; i < nt; i++) {
        if (nnz > 0 && i > 0 && t[i].r == t[i - 1].r && t[i].c == t[i - 1].c) {
            if (g->dense_ybus && t[i].r != t[i].c) {
                /* calcYbus (GPU/sistema.h:673-703, metodo = denso) assigns the
                 * off-diagonal entries branch by branch: the last one stays */
                y->re[nnz - 1] = t[i].re;
                y->im[nnz - 1] = t[i].im;
                continue;
            }
            y->re[nnz - 1] += t[i].re;
            y->im[nnz - 1] += t[i].im;
        } else {
            y->col[nnz] = t[i].c; y->re[nnz] = t[i].re; y->im[nnz] = t[i].im;
            y->rowptr[t[i].r + 1]++;
            nnz++;
        }
    }
    for (int i = 0; i < n; i++) y->rowptr[i + 1] += y->rowptr[i];
    y->nnz = nnz;
    free(t);
    return 0;
}

void orc_ybus_free(orc_ybus *y) {
    free(y->rowptr); free(y->col); free(y->re); free(y->im);
    memset(y, 0, sizeof(*y));
}

static int ypos(const orc_ybus *y, int r, int c) { /* coeffPos, GPU/PQcalc.cuh:23-30 */
    for (int i = y->rowptr[r]; i < y->rowptr[r + 1]; i++) if (y->col[i] == c) return i;
    return -1;
}

/* ------------------------------------------------------------------------- */
/* PQ injections, GPU/PQcalc.cuh:177-219 (same accumulation order)           */
/* ------------------------------------------------------------------------- */
void orc_pq(const orc_ybus *y, const double *V, const double *theta, double *P, double *Q) {
    for (int k = 0; k < y->n; k++) {
        double accp = 0, accq = 0;
        for (int i = y->rowptr[k]; i < y->rowptr[k + 1]; i++) {
            int m = y->col[i];
            double a = theta[k] - theta[m];
            double tp = y->re[i] * cos(a) + y->im[i] * sin(a);
            double tq = y->re[i] * sin(a) - y->im[i] * cos(a);
            accp += tp * V[m];
            accq += tq * V[m];
        }
        P[k] = accp * V[k];
        Q[k] = accq * V[k];
    }
}

/* ------------------------------------------------------------------------- */
/* Jacobian in the reference order                                           */
/* ------------------------------------------------------------------------- */

/* Value of one Jacobian entry, SpCalcH/L/M/N GPU/Jacobiano.cuh:252-344
 * (sub = 'H','N','M','L'; k = row bus, m = column bus, 0-based). */
static double jval(char sub, int k, int m, const orc_ybus *y, const double *V,
                   const double *th, const double *P, const double *Q) {
    int p = ypos(y, k, m);
    double G = y->re[p], B = y->im[p];
    if (k != m) {
        double a = th[k] - th[m];
        switch (sub) {
        case 'H': return V[k] * V[m] * (G * sin(a) - B * cos(a));
        case 'L': return V[k] * (G * sin(a) - B * cos(a));
        case 'M': return -V[k] * V[m] * (G * cos(a) + B * sin(a));
        default:  return V[k] * (G * cos(a) + B * sin(a));
        }
    }
    switch (sub) {
    case 'H': return -Q[k] - V[k] * V[k] * B;
    case 'L': return (Q[k] - V[k] * V[k] * B) / V[k];
    case 'M': return P[k] - V[k] * V[k] * G;
    default:  return (P[k] + V[k] * V[k] * G) / V[k];
    }
}

/* Pattern order of Jstencil0based, GPU/esparso.h:61-178: P rows of the
 * non-slack buses in bus order (H entries, then N entries), then the Q rows of
 * barrasPQlim in list order (M entries, then L entries). */
int orc_jacobian(const orc_grid *g, const orc_ybus *y, const double *V,
                 const double *theta, const double *P, const double *Q,
                 const int *pqlim, int nPQlim,
                 int *dim_out, int *nnz_out, int **rowptr_o, int **col_o, double **val_o) {
    int n = g->nB, s = g->slack - 1;
    int dim = n - 1 + nPQlim;
    int *pqpos = (int *)xcalloc(n, sizeof(int)); /* bus -> position in PQlim, or -1 */
    for (int i = 0; i < n; i++) pqpos[i] = -1;
    for (int i = 0; i < nPQlim; i++) pqpos[pqlim[i] - 1] = i;
    int cap = 4 * y->nnz + 16;
    int *rp = (int *)xcalloc(dim + 1, sizeof(int));
    int *cl = (int *)xcalloc(cap, sizeof(int));
    double *vl = (double *)xcalloc(cap, sizeof(double));
    int nnz = 0, row = 0;
    for (int k = 0; k < n; k++) {
        if (k == s) continue;
        for (int i = y->rowptr[k]; i < y->rowptr[k + 1]; i++) {
            int m = y->col[i];
            if (m == s) continue;
            cl[nnz] = m - (m > s);
            vl[nnz++] = jval('H', k, m, y, V, theta, P, Q);
        }
        for (int i = y->rowptr[k]; i < y->rowptr[k + 1]; i++) {
            int m = y->col[i];
            if (pqpos[m] < 0) continue;
            cl[nnz] = n - 1 + pqpos[m];
            vl[nnz++] = jval('N', k, m, y, V, theta, P, Q);
        }
        rp[++row] = nnz;
    }
    for (int q = 0; q < nPQlim; q++) {
        int k = pqlim[q] - 1;
        for (int i = y->rowptr[k]; i < y->rowptr[k + 1]; i++) {
            int m = y->col[i];
            if (m == s) continue;
            cl[nnz] = m - (m > s);
            vl[nnz++] = jval('M', k, m, y, V, theta, P, Q);
        }
        for (int i = y->rowptr[k]; i < y->rowptr[k + 1]; i++) {
            int m = y->col[i];
            if (pqpos[m] < 0) continue;
            cl[nnz] = n - 1 + pqpos[m];
            vl[nnz++] = jval('L', k, m, y, V, theta, P, Q);
        }
        rp[++row] = nnz;
    }
    free(pqpos);
    *dim_out = dim; *nnz_out = nnz; *rowptr_o = rp; *col_o = cl; *val_o = vl;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Sparse LU: minimum-degree column order + Gilbert-Peierls left-looking LU   */
/* with threshold partial pivoting (diagonal preferred).                      */
/* ------------------------------------------------------------------------- */

typedef struct { int d, v; } hent;
typedef struct { hent *a; int n, cap; } heap_t;
static void hpush(heap_t *h, int d, int v) {
    if (h->n == h->cap) { h->cap = h->cap ? 2 * h->cap : 1024; h->a = (hent *)realloc(h->a, h->cap * sizeof(hent)); }
    int i = h->n++;
    h->a[i].d = d; h->a[i].v = v;
    while (i > 0) {
        int p = (i - 1) / 2;
        if (h->a[p].d < h->a[i].d || (h->a[p].d == h->a[i].d && h->a[p].v <= h->a[i].v)) break;
        hent t = h->a[p]; h->a[p] = h->a[i]; h->a[i] = t; i = p;
    }
}
static hent hpop(heap_t *h) {
    hent r = h->a[0];
    h->a[0] = h->a[--h->n];
    int i = 0;
    for (;;) {
        int l = 2 * i + 1, rr = l + 1, m = i;
        if (l < h->n && (h->a[l].d < h->a[m].d || (h->a[l].d == h->a[m].d && h->a[l].v < h->a[m].v))) m = l;
        if (rr < h->n && (h->a[rr].d < h->a[m].d || (h->a[rr].d == h->a[m].d && h->a[rr].v < h->a[m].v))) m = rr;
        if (m == i) break;
        hent t = h->a[m]; h->a[m] = h->a[i]; h->a[i] = t; i = m;
    }
    return r;
}

/* Minimum degree on the graph of A + A^T, explicit elimination graph. */
static void min_degree(int n, const int *rp, const int *cl, int *order) {
    int **adj = (int **)xcalloc(n, sizeof(int *));
    int *deg = (int *)xcalloc(n, sizeof(int)), *cap = (int *)xcalloc(n, sizeof(int));
    int *w = (int *)xcalloc(n, sizeof(int)), *done = (int *)xcalloc(n, sizeof(int));
    int stamp = 0;
    /* symmetric adjacency without duplicates */
    int *cnt = (int *)xcalloc(n, sizeof(int));
    for (int i = 0; i < n; i++)
        for (int p = rp[i]; p < rp[i + 1]; p++) if (cl[p] != i) { cnt[i]++; cnt[cl[p]]++; }
    for (int i = 0; i < n; i++) { cap[i] = cnt[i] + 4; adj[i] = (int *)xcalloc(cap[i], sizeof(int)); }
    for (int i = 0; i < n; i++)
        for (int p = rp[i]; p < rp[i + 1]; p++) {
            int j = cl[p];
            if (j == i) continue;
            adj[i][deg[i]++] = j;
            adj[j][deg[j]++] = i;
        }
    for (int i = 0; i < n; i++) { /* dedupe */
        stamp++;
        int m = 0;
        w[i] = stamp;
        for (int p = 0; p < deg[i]; p++) { int j = adj[i][p]; if (w[j] != stamp) { w[j] = stamp; adj[i][m++] = j; } }
        deg[i] = m;
    }
    heap_t h = {0};
    for (int i = 0; i < n; i++) hpush(&h, deg[i], i);
    int *nb = (int *)xcalloc(n, sizeof(int));
    int *tmp = NULL, tcap = 0;
    for (int k = 0; k < n; k++) {
        hent e;
        do { e = hpop(&h); } while (done[e.v] || e.d != deg[e.v]);
        int p = e.v;
        order[k] = p;
        done[p] = 1;
        int nn = 0;
        for (int q = 0; q < deg[p]; q++) if (!done[adj[p][q]]) nb[nn++] = adj[p][q];
        for (int a = 0; a < nn; a++) {
            int u = nb[a];
            int need = deg[u] + nn;
            if (need > tcap) { tcap = 2 * need; tmp = (int *)realloc(tmp, tcap * sizeof(int)); }
            stamp++;
            w[u] = stamp;
            int m = 0;
            for (int q = 0; q < deg[u]; q++) { int v = adj[u][q]; if (v != p && !done[v] && w[v] != stamp) { w[v] = stamp; tmp[m++] = v; } }
            for (int q = 0; q < nn; q++) { int v = nb[q]; if (w[v] != stamp) { w[v] = stamp; tmp[m++] = v; } }
            if (m > cap[u]) { cap[u] = 2 * m; adj[u] = (int *)realloc(adj[u], cap[u] * sizeof(int)); }
            memcpy(adj[u], tmp, m * sizeof(int));
            deg[u] = m;
            hpush(&h, m, u);
        }
    }
    for (int i = 0; i < n; i++) free(adj[i]);
    free(adj); free(deg); free(cap); free(w); free(done); free(cnt); free(h.a); free(nb); free(tmp);
}

typedef struct { int *p, *i, cnt, cap; double *x; } cscbuf;
static void cpush(cscbuf *b, int i, double x) {
    if (b->cnt == b->cap) {
        b->cap = b->cap ? 2 * b->cap : 4096;
        b->i = (int *)realloc(b->i, b->cap * sizeof(int));
        b->x = (double *)realloc(b->x, b->cap * sizeof(double));
    }
    b->i[b->cnt] = i; b->x[b->cnt] = x; b->cnt++;
}

int orc_sparse_solve(int n, const int *rowptr, const int *col, const double *val,
                     const double *b, double *xout) {
    if (n == 0) return 0;
    /* CSC of A */
    int nnz = rowptr[n];
    int *cp = (int *)xcalloc(n + 1, sizeof(int)), *ci = (int *)xcalloc(nnz, sizeof(int));
    double *cx = (double *)xcalloc(nnz, sizeof(double));
    for (int p = 0; p < nnz; p++) cp[col[p] + 1]++;
    for (int j = 0; j < n; j++) cp[j + 1] += cp[j];
    int *pos = (int *)xcalloc(n, sizeof(int));
    for (int j = 0; j < n; j++) pos[j] = cp[j];
    for (int r = 0; r < n; r++)
        for (int p = rowptr[r]; p < rowptr[r + 1]; p++) { int q = pos[col[p]]++; ci[q] = r; cx[q] = val[p]; }
    int *q = (int *)xcalloc(n, sizeof(int));
    min_degree(n, rowptr, col, q);

    cscbuf Lb = {0}, Ub = {0};
    Lb.p = (int *)xcalloc(n + 1, sizeof(int));
    Ub.p = (int *)xcalloc(n + 1, sizeof(int));
    int *pinv = (int *)xcalloc(n, sizeof(int));
    for (int i = 0; i < n; i++) pinv[i] = -1;
    double *x = (double *)xcalloc(n, sizeof(double));
    int *mark = (int *)xcalloc(n, sizeof(int)), *stk = (int *)xcalloc(n, sizeof(int));
    int *ptr = (int *)xcalloc(n, sizeof(int)), *topo = (int *)xcalloc(n, sizeof(int));
    int status = 0;
    for (int k = 0; k < n; k++) {
        int j = q[k];
        /* reach of A(:,j) in the graph of L: nodes are rows; a pivotal row r
         * leads to the rows of L(:, pinv[r]).  Output in topological order. */
        int top = n;
        for (int p = cp[j]; p < cp[j + 1]; p++) {
            int r0 = ci[p];
            if (mark[r0] == k + 1) continue;
            int sp = 0;
            stk[0] = r0;
            mark[r0] = k + 1;
            ptr[r0] = pinv[r0] >= 0 ? Lb.p[pinv[r0]] : 0;
            while (sp >= 0) {
                int r = stk[sp];
                int c = pinv[r], advanced = 0;
                if (c >= 0) {
                    int end = Lb.p[c + 1];
                    while (ptr[r] < end) {
                        int r2 = Lb.i[ptr[r]++];
                        if (mark[r2] != k + 1) {
                            mark[r2] = k + 1;
                            ptr[r2] = pinv[r2] >= 0 ? Lb.p[pinv[r2]] : 0;
                            stk[++sp] = r2;
                            advanced = 1;
                            break;
                        }
                    }
                }
                if (!advanced) { sp--; topo[--top] = r; }
            }
        }
        for (int t = top; t < n; t++) x[topo[t]] = 0;
        for (int p = cp[j]; p < cp[j + 1]; p++) x[ci[p]] = cx[p];
        for (int t = top; t < n; t++) {
            int r = topo[t], c = pinv[r];
            if (c < 0) continue;
            double xr = x[r];
            for (int p = Lb.p[c]; p < Lb.p[c + 1]; p++) x[Lb.i[p]] -= Lb.x[p] * xr;
        }
        /* pivot: diagonal row j if within threshold 0.1 of the column maximum */
        int piv = -1;
        double amax = -1;
        for (int t = top; t < n; t++) {
            int r = topo[t];
            if (pinv[r] < 0 && fabs(x[r]) > amax) { amax = fabs(x[r]); piv = r; }
        }
        if (piv < 0 || amax <= 0 || !isfinite(amax)) { status = 2; break; }
        if (pinv[j] < 0 && mark[j] == k + 1 && fabs(x[j]) >= 0.1 * amax) piv = j;
        double pv = x[piv];
        for (int t = top; t < n; t++) {
            int r = topo[t];
            if (pinv[r] >= 0) cpush(&Ub, pinv[r], x[r]);
        }
        cpush(&Ub, k, pv);
        Ub.p[k + 1] = Ub.cnt;
        pinv[piv] = k;
        for (int t = top; t < n; t++) {
            int r = topo[t];
            if (pinv[r] < 0) cpush(&Lb, r, x[r] / pv);
        }
        Lb.p[k + 1] = Lb.cnt;
    }
    if (!status) {
        /* x = Q U^-1 L^-1 P b */
        double *y = (double *)xcalloc(n, sizeof(double));
        for (int i = 0; i < n; i++) y[pinv[i]] = b[i];
        for (int k = 0; k < n; k++) {
            double yk = y[k];
            for (int p = Lb.p[k]; p < Lb.p[k + 1]; p++) y[pinv[Lb.i[p]]] -= Lb.x[p] * yk;
        }
        for (int k = n - 1; k >= 0; k--) {
            int pend = Ub.p[k + 1] - 1; /* diagonal is stored last */
            y[k] /= Ub.x[pend];
            double yk = y[k];
            for (int p = Ub.p[k]; p < pend; p++) y[Ub.i[p]] -= Ub.x[p] * yk;
        }
        for (int k = 0; k < n; k++) xout[q[k]] = y[k];
        free(y);
    }
    free(cp); free(ci); free(cx); free(pos); free(q); free(pinv); free(x); free(mark); free(stk);
    free(ptr); free(topo); free(Lb.p); free(Lb.i); free(Lb.x); free(Ub.p); free(Ub.i); free(Ub.x);
    return status;
}

/* ------------------------------------------------------------------------- */
/* Newton-Raphson driver                                                      */
/* ------------------------------------------------------------------------- */

/* maxi, GPU/newtonRaphson.cuh:24-33 (starts at 0; a NaN never raises it). */
static double maxi(const double *v, int n) {
    double a = 0;
    for (int i = 0; i < n; i++) if (fabs(v[i]) > a) a = fabs(v[i]);
    return a;
}

static void push_event(orc_result *r, int it, int bus, int pvpos, int code) {
    if (r->n_events == r->cap_events) {
        r->cap_events = r->cap_events ? 2 * r->cap_events : 64;
        r->ev_iter = (int *)realloc(r->ev_iter, r->cap_events * sizeof(int));
        r->ev_bus = (int *)realloc(r->ev_bus, r->cap_events * sizeof(int));
        r->ev_pvpos = (int *)realloc(r->ev_pvpos, r->cap_events * sizeof(int));
        r->ev_code = (int *)realloc(r->ev_code, r->cap_events * sizeof(int));
    }
    r->ev_iter[r->n_events] = it; r->ev_bus[r->n_events] = bus;
    r->ev_pvpos[r->n_events] = pvpos; r->ev_code[r->n_events] = code;
    r->n_events++;
}

/* ------------------------------------------------------------------------- */
/* verbose_mode dumps of mNR (GPU/newtonRaphson.cuh:150-156,270-272,284-286,   */
/* 392-427,433-450,539-563; GPU/Jacobiano.cuh:216-220,382-410;                 */
/* GPU/PQcalc.cuh:304-320,417-432) written to vf when it is not NULL.          */
/* ------------------------------------------------------------------------- */
static const char *EV_TEXT[6] = {"", "PV -> PQ (limite superior)", "PQ (limite inferior) -> PQ (limite superior)",
                                 "PV -> PQ (limite inferior)", "PQ (limite superior) -> PQ (limite inferior)",
                                 "PQ -> PV"};

/* showVec, GPU/dim.h:11-37 (fixed, prec decimals); "[]" for an empty vector */
static void vshow(FILE *f, const double *v, int n, int prec) {
    if (n <= 0) { fputs("[]\n", f); return; }
    fprintf(f, "[%.*f\n", prec, v[0]);
    for (int i = 1; i < n - 1; i++) fprintf(f, " %.*f\n", prec, v[i]);
    fprintf(f, " %.*f]\n", prec, v[n - 1]);
}
static void vshowi(FILE *f, const int *v, int n) {
    if (n <= 0) { fputs("[]\n", f); return; }
    fprintf(f, "[%d\n", v[0]);
    for (int i = 1; i < n - 1; i++) fprintf(f, " %d\n", v[i]);
    fprintf(f, " %d]\n", v[n - 1]);
}

/* the lists and limits block printed by printAlLim (GPU/limiteInjReat.cuh:226-242)
 * and, with a leading blank line each, by mNR after the mismatch (:399-414) */
static void vlists(FILE *f, const orc_grid *g, const int *limQ, const int *pvlim, int nPVlim, const int *pqlim,
                   int nPQlim, const double *QliqLim, const char *sep) {
    fprintf(f, "%slimQ:\n", sep);
    vshowi(f, limQ, g->nPV);
    fprintf(f, "%sbarrasPVlim:\n", sep);
    vshowi(f, pvlim, nPVlim);
    fprintf(f, "%sbarrasPQlim:\n", sep);
    vshowi(f, pqlim, nPQlim);
    fprintf(f, "%slimQinf:\n", sep);
    vshow(f, g->Qmin, g->nPV, 4);
    fprintf(f, "%slimQsup:\n", sep);
    vshow(f, g->Qmax, g->nPV, 4);
    fprintf(f, "%sQliqLim:\n", sep);
    vshow(f, QliqLim, g->nB, 4);
}

static int solve_impl(const orc_grid *g, const orc_opts *o, orc_result *r, FILE *vf);

int orc_solve(const orc_grid *g, const orc_opts *o, orc_result *r) { return solve_impl(g, o, r, NULL); }

int orc_solve_verbose(const orc_grid *g, const orc_opts *o, orc_result *r, void *out) {
    return solve_impl(g, o, r, (FILE *)out);
}

static int solve_impl(const orc_grid *g, const orc_opts *o, orc_result *r, FILE *vf) {
    memset(r, 0, sizeof(*r));
    int n = g->nB, nPV = g->nPV, nPQ = g->nPQ, s = g->slack - 1;
    orc_ybus y;
    orc_build_ybus(g, &y);
    double *V = (double *)xcalloc(n, sizeof(double)), *th = (double *)xcalloc(n, sizeof(double));
    double *P = (double *)xcalloc(n, sizeof(double)), *Q = (double *)xcalloc(n, sizeof(double));
    memcpy(V, g->V, n * sizeof(double));
    memcpy(th, g->theta, n * sizeof(double));
    /* initLim, GPU/limiteInjReat.cuh:188-224 */
    int *pqlim = (int *)xcalloc(nPV + nPQ, sizeof(int));
    int *limQ = (int *)xcalloc(nPV, sizeof(int));
    double *QliqLim = (double *)xcalloc(n, sizeof(double));
    memcpy(pqlim, g->barrasPQ, nPQ * sizeof(int));
    int nPQlim = nPQ, nPVlim = nPV;
    memcpy(QliqLim, g->Qliq, n * sizeof(double));
    int ngLim = 2 * nPQ + nPV;
    double *gl = (double *)xcalloc(2 * (nPV + nPQ) + 1, sizeof(double)); /* gLim */
    double *dx = (double *)xcalloc(2 * (nPV + nPQ) + 1, sizeof(double));
    r->hist = (double *)xcalloc(o->no_max_iter + 1, sizeof(double));
    int it, converged = 0, status = 0;
    double maxG = 0;
    int *pvlim = (int *)xcalloc(nPV + 1, sizeof(int));
    double *prevJ = NULL; /* the Jacobian value array as the last fill left it (NULL: a new, zeroed stencil) */
    int prevN = 0;
    memcpy(pvlim, g->barrasPV, nPV * sizeof(int));
    if (vf && o->lim_inj_reat) {
        fprintf(vf, "nPQlim = %d\nnPVlim = %d\n", nPQlim, nPVlim);
        vlists(vf, g, limQ, pvlim, nPVlim, pqlim, nPQlim, QliqLim, "");
    }
    for (it = 0; it < o->no_max_iter; it++) {
        if (vf)
            fprintf(vf, "\n****************************************************************** ITERACAO %d "
                        "******************************************************************\n", it);
        orc_pq(&y, V, th, P, Q);
        if (vf && g->dense_ybus) {
            for (int k = 0; k < n; k++) fprintf(vf, "P_%d\t= %f\n", k + 1, P[k]);
            for (int k = 0; k < n; k++) fprintf(vf, "Q_%d\t= %f\n", k + 1, Q[k]);
        }
        /* limit trigger on the previous step, GPU/newtonRaphson.cuh:309-384 */
        if (it >= 1 && o->lim_inj_reat && maxi(dx, ngLim) < o->tol * 10.) {
            /* chkLimQ, GPU/limiteInjReat.cuh:5-40 */
            int ev0 = r->n_events;
            for (int i = 0; i < nPV; i++) {
                int b = g->barrasPV[i] - 1;
                double qg = Q[b] + g->Qload[b];
                if (qg < g->Qmin[i] - o->tol) {
                    if (!limQ[i]) push_event(r, it, b + 1, i, ORC_EV_PV_TO_PQ_MIN);
                    else if (QliqLim[b] != g->Qmin[i] - g->Qload[b]) push_event(r, it, b + 1, i, ORC_EV_PQMAX_TO_PQMIN);
                    limQ[i] = 1;
                    QliqLim[b] = g->Qmin[i] - g->Qload[b];
                } else if (qg > g->Qmax[i] + o->tol) {
                    if (!limQ[i]) push_event(r, it, b + 1, i, ORC_EV_PV_TO_PQ_MAX);
                    else if (QliqLim[b] != g->Qmax[i] - g->Qload[b]) push_event(r, it, b + 1, i, ORC_EV_PQMIN_TO_PQMAX);
                    limQ[i] = 1;
                    QliqLim[b] = g->Qmax[i] - g->Qload[b];
                } else {
                    if (limQ[i]) push_event(r, it, b + 1, i, ORC_EV_PQ_TO_PV);
                    limQ[i] = 0;
                }
            }
            /* geraVetPV / geraVetPQ, GPU/limiteInjReat.cuh:42-75: ascending merge */
            nPVlim = 0;
            for (int i = 0; i < nPV; i++) if (!limQ[i]) nPVlim++;
            int a = 0, c = 0;
            for (int i = 0; i < nPV; i++) {
                if (!limQ[i]) continue;
                while (a < nPQ && g->barrasPQ[a] < g->barrasPV[i]) pqlim[c++] = g->barrasPQ[a++];
                pqlim[c++] = g->barrasPV[i];
            }
            while (a < nPQ) pqlim[c++] = g->barrasPQ[a++];
            nPQlim = c;
            ngLim = nPQlim + nPQlim + nPVlim;
            c = 0;
            for (int i = 0; i < nPV; i++) if (!limQ[i]) pvlim[c++] = g->barrasPV[i];
            if (vf) {
                fputs("\n", vf);
                for (int e = ev0; e < r->n_events; e++)
                    fprintf(vf, "Barra %d [%d]: %s\n", r->ev_bus[e], r->ev_pvpos[e], EV_TEXT[r->ev_code[e]]);
            }
            free(prevJ); /* Jstencil0based + d_attSparse: new stencil, values zeroed */
            prevJ = NULL;
        }
        /* calcResPLim / calcResQLim, GPU/newtonRaphson.cuh:35-58 */
        int m = 0;
        for (int k = 0; k < n; k++) if (k != s) gl[m++] = g->Pliq[k] - P[k];
        for (int i = 0; i < nPQlim; i++) { int b = pqlim[i] - 1; gl[m++] = QliqLim[b] - Q[b]; }
        maxG = maxi(gl, ngLim);
        r->hist[r->n_hist++] = maxG;
        if (vf) {
            fprintf(vf, "Pcalc^(%d) =\n", it);
            vshow(vf, P, n, 4);
            fprintf(vf, "\nQcalc^(%d) =\n", it);
            vshow(vf, Q, n, 4);
            fprintf(vf, "\ndeltaP^(%d) =\n", it);
            vshow(vf, gl, n - 1, 4);
            fprintf(vf, "\ndeltaQ^(%d) =\n", it);
            vshow(vf, gl + n - 1, nPQlim, 4);
            vlists(vf, g, limQ, pvlim, nPVlim, pqlim, nPQlim, QliqLim, "\n");
            fprintf(vf, "\nmax(g) = %e", maxG);
        }
        if (maxG <= o->tol) { /* :421-426 */
            if (vf) fprintf(vf, "\n\nbreak!\nmax(g) = %e\n\n", maxG);
            converged = 1;
            break;
        }
        if (vf) fputs("     ...     continua:\n\n", vf);
        int dim, nnz, *rp, *cl;
        double *vl;
        orc_jacobian(g, &y, V, th, P, Q, pqlim, nPQlim, &dim, &nnz, &rp, &cl, &vl);
        if (vf && g->dense_ybus) { /* calcJacLim's JacobianoN, showMat GPU/dim.h:157-167 */
            fputs("JacobianoN =\n\n[", vf);
            for (int i = 0; i < dim; i++) {
                int p = rp[i];
                for (int j = 0; j < dim; j++) {
                    double a = 0;
                    if (p < rp[i + 1] && cl[p] == j) a = vl[p++];
                    fprintf(vf, "%5.1f ", a);
                }
                fputs("\n ", vf);
            }
            fputs("]\n\n", vf);
        } else if (vf) { /* SpCalcJac: H, L, M filled in turn, the array printed after each */
            double *cur = (double *)xcalloc(nnz + 1, sizeof(double));
            if (prevJ && prevN == nnz) memcpy(cur, prevJ, nnz * sizeof(double));
            const char *name[3] = {"H", "L", "M"};
            for (int part = 0; part < 3; part++) {
                for (int i = 0; i < dim; i++)
                    for (int p = rp[i]; p < rp[i + 1]; p++) {
                        int prow = i < n - 1, pcol = cl[p] < n - 1;
                        if (part == 0 ? (prow && pcol) : part == 1 ? (!prow && !pcol) : (!prow && pcol)) cur[p] = vl[p];
                    }
                fprintf(vf, "%s^(%d) =\n", name[part], it);
                vshow(vf, cur, nnz, 5);
            }
            free(cur);
            fprintf(vf, "J^(%d) =\n", it);
            vshow(vf, vl, nnz, 5);
            free(prevJ);
            prevJ = (double *)xcalloc(nnz + 1, sizeof(double));
            memcpy(prevJ, vl, nnz * sizeof(double));
            prevN = nnz;
        }
        if (vf) {
            fprintf(vf, "V^(%d) = \n", it);
            vshow(vf, V, n, 5);
            fprintf(vf, "theta^(%d) = \n", it);
            vshow(vf, th, n, 5);
            fputs("deltaPQ = \n", vf);
            vshow(vf, gl, ngLim, 5);
        }
        status = orc_sparse_solve(dim, rp, cl, vl, gl, dx);
        free(rp); free(cl); free(vl);
        if (status) break;
        if (vf) {
            fprintf(vf, "\n (deltaX)g^(%d) = \n", it);
            vshow(vf, dx, ngLim, 5);
        }
        /* attOlim / attVlim, GPU/newtonRaphson.cuh:76-100 */
        m = 0;
        for (int k = 0; k < n; k++) if (k != s) th[k] += dx[m++];
        for (int i = 0; i < nPQlim; i++) V[pqlim[i] - 1] += dx[n - 1 + i];
        if (vf) {
            fprintf(vf, "V^(%d) = \n", it + 1);
            vshow(vf, V, n, 6);
            fprintf(vf, "theta^(%d) = \n", it + 1);
            vshow(vf, th, n, 6);
        }
    }
    free(prevJ);
    free(pvlim);
    if (!converged && !status) it = o->no_max_iter;
    r->status = status;
    r->converged = converged;
    r->iterations = it;
    r->final_mismatch = maxG;
    r->nPQlim = nPQlim;
    r->limQ = limQ;
    r->V = V; r->theta = th; r->Pcalc = P; r->Qcalc = Q;
    r->Pdp = (double *)xcalloc(g->nL, sizeof(double));
    r->Ppd = (double *)xcalloc(g->nL, sizeof(double));
    r->Qdp = (double *)xcalloc(g->nL, sizeof(double));
    r->Qpd = (double *)xcalloc(g->nL, sizeof(double));
    orc_flows(g, &y, V, th, r->Pdp, r->Ppd, r->Qdp, r->Qpd);
    free(pqlim); free(QliqLim); free(gl); free(dx);
    orc_ybus_free(&y);
    return status;
}

void orc_result_free(orc_result *r) {
    free(r->hist); free(r->ev_iter); free(r->ev_bus); free(r->ev_pvpos); free(r->ev_code);
    free(r->limQ); free(r->V); free(r->theta); free(r->Pcalc); free(r->Qcalc);
    free(r->Pdp); free(r->Ppd); free(r->Qdp); free(r->Qpd);
    memset(r, 0, sizeof(*r));
}

/* ------------------------------------------------------------------------- */
/* Branch flows, d_P_Eficiente_Sp / d_Q_Eficiente_Sp GPU/PQcalc.cuh:523-545,  */
/* with phif GPU/PQcalc.cuh:32-46 and bshf GPU/PQcalc.cuh:81-97.              */
/* ------------------------------------------------------------------------- */
void orc_flows(const orc_grid *g, const orc_ybus *y, const double *V,
               const double *theta, double *Pdp, double *Ppd, double *Qdp, double *Qpd) {
    for (int b = 0; b < g->nL; b++) {
        int k = g->de[b], m = g->para[b];
        /* phif(k, m): phase of branch (k,m), else minus that of (m,k), else 0 */
        double ph = 0;
        int found = 0;
        for (int i = 0; i < g->nL; i++) if (g->de[i] == k && g->para[i] == m) { ph = g->phi[i]; found = 1; break; }
        if (!found)
            for (int i = 0; i < g->nL; i++) if (g->de[i] == m && g->para[i] == k) { ph = -g->phi[i]; break; }
        double a = ph + theta[k - 1] - theta[m - 1];
        double bkm = 0, bmk = 0;
        for (int i = 0; i < g->nL; i++) {
            if ((g->de[i] == k && g->para[i] == m) || (g->de[i] != k && g->para[i] == k && g->de[i] == m)) { bkm = g->bsh_br[i]; break; }
        }
        for (int i = 0; i < g->nL; i++) {
            if ((g->de[i] == m && g->para[i] == k) || (g->de[i] != m && g->para[i] == m && g->de[i] == k)) { bmk = g->bsh_br[i]; break; }
        }
        int pkm = ypos(y, k - 1, m - 1), pmk = ypos(y, m - 1, k - 1);
        double Gkm = y->re[pkm], Bkm = y->im[pkm], Gmk = y->re[pmk], Bmk = y->im[pmk];
        double Vk = V[k - 1], Vm = V[m - 1];
        Pdp[b] = Vk * Vk * Gkm - Vk * Vm * Gkm * cos(a) - Vk * Vm * Bkm * sin(a);
        Ppd[b] = Vm * Vm * Gmk - Vm * Vk * Gmk * cos(-a) - Vm * Vk * Bmk * sin(-a);
        Qdp[b] = -Vk * Vk * (Bkm + bkm) + Vk * Vm * Bkm * cos(a) - Vk * Vm * Gkm * sin(a);
        Qpd[b] = -Vm * Vm * (Bmk + bmk) + Vm * Vk * Bmk * cos(-a) - Vm * Vk * Gmk * sin(-a);
    }
}
