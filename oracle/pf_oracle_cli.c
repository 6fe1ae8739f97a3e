/*
 * pf_oracle_cli.c -- command-line driver of the CPU oracle (test infrastructure
 * only).  Solves one grid and prints a JSON summary; with --repeat N it solves
 * N times and reports the wall time per solve, for the CPU-baseline figure;
 * with --verbose it prints the reference's verbose_mode dumps of the solve
 * instead (--dense: the Ybus rule and dumps of metodo = denso).
 *
 *   pforacle <file.cdf|.cdfx|.m> [--tol T] [--maxit N] [--lim 0|1] [--repeat N] [--state]
 *            [--verbose] [--dense]
 */
#define _POSIX_C_SOURCE 199309L
#include "pf_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static double now(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: pforacle <file> [--tol T] [--maxit N] [--lim 0|1] [--repeat N] [--state]\n");
        return 2;
    }
    orc_opts o = {1.0, 0.0, 1e-8, 100, 0};
    int repeat = 1, state = 0, verbose = 0, dense = 0;
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "--tol") && i + 1 < argc) o.tol = atof(argv[++i]);
        else if (!strcmp(argv[i], "--maxit") && i + 1 < argc) o.no_max_iter = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--lim") && i + 1 < argc) o.lim_inj_reat = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--repeat") && i + 1 < argc) repeat = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--state")) state = 1;
        else if (!strcmp(argv[i], "--verbose")) verbose = 1;
        else if (!strcmp(argv[i], "--dense")) dense = 1;
    }
    char err[256];
    orc_grid g;
    double t0 = now();
    const size_t len = strlen(argv[1]);
    const int is_m = len > 2 && !strcmp(argv[1] + len - 2, ".m");
    if ((is_m ? orc_read_m : orc_read_cdf)(argv[1], o.v_inicial, o.theta_inicial, &g, err, sizeof err)) {
        fprintf(stderr, "pforacle: %s\n", err);
        return 1;
    }
    double t1 = now();
    g.dense_ybus = dense;
    if (verbose) {
        orc_result rv;
        orc_solve_verbose(&g, &o, &rv, stdout);
        orc_result_free(&rv);
        orc_grid_free(&g);
        return 0;
    }
    orc_result r;
    memset(&r, 0, sizeof r);
    double ts = now();
    for (int k = 0; k < repeat; k++) {
        if (k) orc_result_free(&r);
        orc_solve(&g, &o, &r);
    }
    double te = now();
    printf("{\"file\": \"%s\", \"nB\": %d, \"nL\": %d, \"nPV\": %d, \"nPQ\": %d, ", argv[1], g.nB, g.nL, g.nPV, g.nPQ);
    printf("\"status\": %d, \"converged\": %d, \"iterations\": %d, \"final_mismatch\": %.17g, ",
           r.status, r.converged, r.iterations, r.final_mismatch);
    printf("\"n_events\": %d, \"read_s\": %.6f, \"solve_s\": %.9f, \"repeat\": %d",
           r.n_events, t1 - t0, (te - ts) / repeat, repeat);
    if (state) {
        printf(", \"V\": [");
        for (int i = 0; i < g.nB; i++) printf("%s%.17g", i ? ", " : "", r.V[i]);
        printf("], \"theta\": [");
        for (int i = 0; i < g.nB; i++) printf("%s%.17g", i ? ", " : "", r.theta[i]);
        printf("]");
    }
    printf("}\n");
    orc_result_free(&r);
    orc_grid_free(&g);
    return 0;
}
