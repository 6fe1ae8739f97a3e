/*
 * gbpf.h -- C ABI of libgbpf, a GB300 (sm_103a) Newton-Raphson AC power-flow
 * engine that is a drop-in for the solve path of
 * joaovdd/Experience-of-Using-GPU-in-Power-Flow-Computation (GPU/ tree).
 *
 * The reference has no library interface: its boundary is the process
 * (data.txt options + a common-data-format file in, a per-bus table and limit
 * lines out) with the in-process call chain
 *     loadFile()                      GPU/sistInfo.h:62-242
 *  -> lerArquivoEAlocarMemoria()      GPU/arquivo.h:250-295
 *  -> calcYbusSp_eficinte()           GPU/sistema.h:705-758
 *  -> mNR()                           GPU/newtonRaphson.cuh:171-623
 *  -> calcFluxf_Eficiente_Sp()        GPU/PQcalc.cuh:547-557
 *  -> impressao2()                    GPU/impressao.h:47-80
 * Each entry point below names the reference step it replaces.
 *
 * Conventions: plain C types only; the caller owns every host buffer; the
 * library owns every device allocation; no entry point prints or exits; every
 * entry point returns a gbpf_status.  One solver handle owns one CUDA stream
 * and is not thread-safe; different handles may be used from different host
 * threads.  Bus indices are 1-based in file order, as in the reference.
 */
#ifndef GBPF_H
#define GBPF_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBPF_ABI_VERSION 1

typedef enum {
    GBPF_OK = 0,
    GBPF_E_INPUT = 1,       /* malformed data.txt / CDF, inconsistent arrays      */
    GBPF_E_SINGULAR = 2,    /* zero or non-finite pivot in the Jacobian LU        */
    GBPF_E_NOCONV = 3,      /* no_max_iter reached with max|g| > tolerancia       */
    GBPF_E_CUDA = 4,        /* CUDA runtime error (message via gbpf_last_error)   */
    GBPF_E_TIMEOUT = 5,     /* a bounded device wait ran out                      */
    GBPF_E_OOM = 6,         /* device or host allocation failed                   */
    GBPF_E_ARG = 7,         /* NULL handle, bad size, buffer too small            */
    GBPF_E_UNSUPPORTED = 8  /* option or input format outside the supported path */
} gbpf_status;

/* metodo values of data.txt (GPU/sistInfo.h:11-17, :89-118). */
typedef enum {
    GBPF_METODO_ESPARSO = 0,
    GBPF_METODO_DENSO = 1,
    GBPF_METODO_HIBRIDOA = 2,
    GBPF_METODO_HIBRIDOB = 3,
    GBPF_METODO_HIBRIDOC = 4,
    GBPF_METODO_NDA = 5
} gbpf_metodo;

/* output_bench values (GPU/sistInfo.h:31-35, :190-203). */
typedef enum { GBPF_BENCH_ALL = 0, GBPF_BENCH_SCREEN = 1, GBPF_BENCH_FILE = 2 } gbpf_output_bench;

/* Branch stamps of a grid's Ybus.  GBPF_YBUS_CDF: calcYbusSp_eficinte
 * (GPU/sistema.h:705-758), the line charging b/2 added undivided on both
 * sides.  GBPF_YBUS_MATPOWER: calcYbusSp_Matpower (GPU/sistema.h:760-855),
 * chosen by the reference for .m input (GPU/main.cu:78-81): the from-side
 * term (1/z + j b/2) divided by |tap|^2.  metodo = denso always uses calcYbus
 * (GPU/sistema.h:673-703), whose stamps are the CDF form. */
typedef enum { GBPF_YBUS_CDF = 0, GBPF_YBUS_MATPOWER = 1 } gbpf_ybus_form;

/* Numeric form of the linear solve (not a data.txt key of the reference). */
typedef enum {
    GBPF_PREC_FP64 = 0,       /* FP64 LU and triangular solves (oracle-matching) */
    GBPF_PREC_FP32_IR = 1     /* FP32 LU and triangular solves + FP64 refinement  */
} gbpf_precision;

/* How gbpf_solve runs the Newton loop (not a data.txt key of the reference;
 * both replace the host loop of mNR, GPU/newtonRaphson.cuh:283-565).
 * GRAPH: one CUDA graph whose device-side WHILE node repeats the iteration's
 * kernels (injections, limits, mismatch, fill, factor, substitutions,
 * update), each phase spread over the whole GPU.  PERSISTENT: the whole loop
 * as one launch of one thread block (the batch's block-per-instance kernel on
 * the solver's own arrays), for grids whose state fits a block's shared
 * memory: no per-phase launches, so a small grid's solve is bound by its own
 * dependent latency only. */
typedef enum { GBPF_FORM_GRAPH = 1, GBPF_FORM_PERSISTENT = 2 } gbpf_form;

/* The data.txt options, namespace global of GPU/sistInfo.h:37-60, with the
 * same defaults. */
typedef struct {
    int metodo;                 /* gbpf_metodo */
    double v_inicial;           /* 1.0 */
    double theta_inicial;       /* 0.0 */
    double tolerancia;          /* 1e-4 */
    int no_max_iter;            /* 100 */
    int lim_inj_reat;           /* 0 */
    int openmp;                 /* 1 */
    int laconic_mode;           /* 0 */
    int verbose_mode;           /* 0 */
    int output_ans;             /* 1 */
    int output_iter;            /* 0  (output_processo_iterativo) */
    int streams;                /* 1 */
    int output_bench;           /* gbpf_output_bench, GBPF_BENCH_ALL */
    int precision;              /* gbpf_precision, GBPF_PREC_FP64 */
    char arq_entrada[1024];     /* "ieee14.cdf" */
} gbpf_options;

/* Fills *o with the defaults of GPU/sistInfo.h:37-60. */
gbpf_status gbpf_options_default(gbpf_options *o);

/* loadFile (GPU/sistInfo.h:62-242) over the text of a data.txt, with the same
 * key lookup (first occurrence of the key name, value between '=' and ';') and
 * the same handling of absent keys.  The lines the reference echoes when
 * laconic_mode is OFF are written to echo (may be NULL). */
gbpf_status gbpf_options_parse(const char *text, gbpf_options *o, char *echo, size_t echo_cap);

/* Same, reading the file at path (the reference reads "data.txt" from the
 * working directory). */
gbpf_status gbpf_options_load(const char *path, gbpf_options *o, char *echo, size_t echo_cap);

/* ------------------------------------------------------------------------ */
/* Grids: struct sistema / barra / ramo of GPU/sistema.h:24-126              */
/* ------------------------------------------------------------------------ */

typedef struct gbpf_grid gbpf_grid;

/* lerArquivoEAlocarMemoria (GPU/arquivo.h:250-295): .cdf (GPU/sistema.h:
 * 386-638), .cdfx (GPU/arquivo.h:4-248) and MATPOWER .m (GPU/m.h:296-622;
 * such a grid gets GBPF_YBUS_MATPOWER).  Buses start at v_inicial /
 * theta_inicial except PV and slack voltages and the slack angle, which come
 * from the file.  Notices the reference prints while reading (parallel
 * branches whose taps differ, PV or slack buses without a generator row) are
 * written to msg. */
gbpf_status gbpf_grid_read(const char *path, double v_inicial, double theta_inicial,
                           gbpf_grid **out, char *msg, size_t msg_cap);

/* A grid from caller arrays (already-merged branches, 1-based bus indices).
 * bus_type: 0/1 = PQ, 2 = PV, 3 = slack (exactly one).  Qmax/Qmin are per bus
 * in p.u. (read for PV buses only).  V0 / theta0 are the starting state. */
typedef struct {
    int nB, nL;
    double baseMVA;
    const int *id, *bus_type;
    const double *V0, *theta0, *Pload, *Qload, *Pg, *Qg, *gsh, *bsh, *Qmax, *Qmin;
    const int *from_bus, *to_bus;
    const double *r, *x, *bch, *tap_re, *tap_im, *phase;
} gbpf_grid_desc;
gbpf_status gbpf_grid_create(const gbpf_grid_desc *d, gbpf_grid **out);

void gbpf_grid_free(gbpf_grid *g);

/* dims[0..7] = nB, nL, nPV, nPQ, slack (1-based), nnzY, baseMVA, notices. */
gbpf_status gbpf_grid_dims(const gbpf_grid *g, int dims[8]);

/* Copies of the bus arrays ([nB] each; any pointer may be NULL). */
gbpf_status gbpf_grid_buses(const gbpf_grid *g, int *id, int *type, double *V0, double *theta0,
                            double *Pload, double *Qload, double *Pg, double *Qg,
                            double *gsh, double *bsh);
/* PV list with limits and setpoints ([nPV]) and PQ list ([nPQ]), 1-based. */
gbpf_status gbpf_grid_pvpq(const gbpf_grid *g, int *pv, double *Qmin, double *Qmax,
                           double *Vset, int *pq);
/* Branch arrays ([nL]). */
gbpf_status gbpf_grid_branches(const gbpf_grid *g, int *from_bus, int *to_bus, double *r,
                               double *x, double *bch, double *tap_re, double *tap_im,
                               double *phase);

/* Replace loads, generation and the starting state of a grid (a scenario);
 * NULL leaves an array unchanged.  Net injections are recomputed as
 * Pg - Pload, Qg - Qload (GPU/sistema.h:546-547). */
gbpf_status gbpf_grid_set_buses(gbpf_grid *g, const double *Pload, const double *Qload,
                                const double *Pg, const double *Qg, const double *V0,
                                const double *theta0);

/* Writes the grid as a fixed-column common-data-format file that the reader
 * above (and the reference's readCDF) reads back. */
gbpf_status gbpf_grid_write_cdf(const gbpf_grid *g, const char *path, const char *title);

/* Writes the grid as a MATPOWER case (version 2, tab-separated rows of 13 bus,
 * 21 generator and 13 branch columns) that the reader above and the
 * reference's lerArquivoMatPOWEReficiente read back.  Values are printed with
 * 17 significant digits.  Generation at a PQ bus is written as negative load,
 * because the reference's .m reader looks generators up for PV and slack
 * buses only (GPU/m.h:310-357). */
gbpf_status gbpf_grid_write_m(const gbpf_grid *g, const char *path, const char *title);

/* The grid's Ybus form (gbpf_ybus_form); the setter lets a grid built by
 * gbpf_grid_create take the MATPOWER form. */
int gbpf_grid_ybus_form(const gbpf_grid *g);
gbpf_status gbpf_grid_set_ybus_form(gbpf_grid *g, int form);

/* Seeded synthetic grids (no counterpart in the reference, which ships IEEE
 * cases only): kind 1 = 14-bus ring-plus-chords grid, 2 = 118-bus meshed grid,
 * 3 = `tiles` copies of kind 2 tied into one grid (128 -> 15,104 buses,
 * 16 -> 1,888 buses), 4 = a kind-1-style grid scaled to `nbus` buses. */
gbpf_status gbpf_generate(int kind, unsigned long long seed, int tiles, int nbus, gbpf_grid **out);

/* Host-only symbolic analysis of the Newton Jacobian of a grid (the part of
 * gbpf_solver_create that needs no GPU): info[0..7] = blocks (nB-1), factor
 * blocks per triangle, update pairs, forward levels, backward levels, Ybus
 * nonzeros, Jacobian block nonzeros, 1 when every update target exists in
 * the factor pattern (closure check). */
gbpf_status gbpf_grid_analyse(const gbpf_grid *g, long long info[8]);

/* ------------------------------------------------------------------------ */
/* Solver: mNR (GPU/newtonRaphson.cuh:171-623) on one GPU                    */
/* ------------------------------------------------------------------------ */

typedef struct gbpf_solver gbpf_solver;

/* Builds everything that depends only on topology, once: the Ybus pattern
 * and its device assembly (replaces calcYbusSp_eficinte), the fixed Jacobian
 * block pattern with room for every PV bus (replaces Jstencil_eficiente /
 * Jstencil0based, GPU/esparso.h:61-178,481-654), the fill-reducing ordering,
 * the symbolic LU and its level schedule, and the CUDA graph of the Newton
 * loop.  device = CUDA ordinal. */
gbpf_status gbpf_solver_create(const gbpf_grid *g, const gbpf_options *o, int device,
                               gbpf_solver **out);
void gbpf_solver_free(gbpf_solver *s);

typedef struct {
    int status;             /* gbpf_status of the solve */
    int converged;          /* 1 when max|g| <= tolerancia */
    int iterations;         /* iterPon.iteracao at return (GPU/newtonRaphson.cuh:283,425) */
    int n_events;           /* PV/PQ switch events recorded */
    int nPQlim;             /* PQ buses at the end (original PQ + PV at a limit) */
    double final_mismatch;  /* max|g| of the returned state */
} gbpf_result;

/* One solve from the grid's starting state (copied to the device at solver
 * creation or by gbpf_solver_set_start).  One graph launch, one host sync. */
gbpf_status gbpf_solve(gbpf_solver *s, gbpf_result *r);

/* Starting state and injections for the next solve, from host arrays [nB]
 * (any may be NULL = unchanged).  Copies host -> device on the solver stream. */
gbpf_status gbpf_solver_set_start(gbpf_solver *s, const double *V0, const double *theta0,
                                  const double *Pliq, const double *Qliq);

/* Results of the last solve, device -> host: state and injections [nB]. */
gbpf_status gbpf_solver_state(gbpf_solver *s, double *V, double *theta, double *Pcalc,
                              double *Qcalc);
/* Switch events of the last solve, 4 ints each: iteration, bus (1-based),
 * PV position, code (1..5, the five chkLimQ lines of GPU/limiteInjReat.cuh:
 * 12,15,23,26,34).  *n = events copied. */
gbpf_status gbpf_solver_events(gbpf_solver *s, int *ev, int cap, int *n);
/* max|g| per iteration of the last solve; *n = entries copied. */
gbpf_status gbpf_solver_history(gbpf_solver *s, double *hist, int cap, int *n);
/* Per iteration of the last solve, 1 where the reactive-limit check ran (the
 * trigger of GPU/newtonRaphson.cuh:309-314 fired); *n = entries copied. */
gbpf_status gbpf_solver_triggers(gbpf_solver *s, int *trig, int cap, int *n);
/* Branch flows of the last solve [nL] (calcFluxf_Eficiente_Sp,
 * GPU/PQcalc.cuh:523-557, computed on the device). */
gbpf_status gbpf_solver_flows(gbpf_solver *s, double *Pdp, double *Ppd, double *Qdp, double *Qpd);

/* Iteration trace: the intermediate values the reference prints when
 * verbose_mode = ON (GPU/newtonRaphson.cuh:150-156,270-272,284-286,392-427,
 * 433-450,539-563; GPU/Jacobiano.cuh:216-220,382-410).  One record per stage
 * of each Newton iteration, in the order the reference's loop reaches them. */
typedef enum {
    GBPF_TRACE_EVAL = 0,     /* injections, the reactive-limit check (when its
                              * trigger fired) and the mismatch, with the
                              * convergence test's outcome */
    GBPF_TRACE_JACOBIAN = 1, /* the Jacobian at the current state; g is still
                              * the mismatch */
    GBPF_TRACE_STEP = 2,     /* the Newton step: g holds dx */
    GBPF_TRACE_UPDATE = 3    /* the state after the update */
} gbpf_trace_stage;

typedef struct {
    int stage;                 /* gbpf_trace_stage */
    int iteration;             /* iterPon.iteracao */
    int nB, nPV, nPQlim, nPVlim;
    int done, converged;       /* EVAL: the loop ends here / converged */
    double max_g;              /* EVAL: max|g| */
    int limit_check;           /* EVAL: 1 when chkLimQ ran in this iteration */
    int n_events;              /* EVAL: switches of this iteration's check, */
    const int *events;         /* 4 ints each as gbpf_solver_events */
    const double *P, *Q;       /* [nB] injections at the current state */
    const double *V, *theta;   /* [nB] the current state */
    const double *QliqLim;     /* [nB] */
    const int *limQ;           /* [nPV] 1 = PV bus held at a Q limit */
    const int *pv_lim;         /* barrasPVlim [nPVlim], 1-based buses */
    const int *pq_lim;         /* barrasPQlim [nPQlim], 1-based, ascending */
    int n_g;                   /* nB - 1 + nPQlim */
    const double *g;           /* EVAL, JACOBIAN: mismatch gLim; STEP: dx;
                                * in the reference's numbering (P rows of the
                                * non-slack buses in bus order, then Q rows in
                                * barrasPQlim order) */
    int nnzJ;                  /* JACOBIAN: entries, in the reference's CSR */
    const int *jrow, *jcol;    /* order (rows, then columns, ascending; */
    const double *jval;        /* 0-based, same numbering as g) */
} gbpf_trace;

typedef void (*gbpf_trace_fn)(const gbpf_trace *t, void *user);

/* A solve that stops after every stage of every iteration, copies the
 * device state to host buffers and calls fn(record, user); the arrays are
 * valid during the call only.  Runs the graph form's kernels one stage at a
 * time (one host synchronisation per stage, for inspection, not speed), so
 * iterations, switch events, state and flows are those of the graph form;
 * gbpf_solver_state / _events / _history / _flows read its results
 * afterwards.  Used by the gbpf driver for verbose_mode = ON. */
gbpf_status gbpf_solve_traced(gbpf_solver *s, gbpf_result *r, gbpf_trace_fn fn, void *user);

/* How the LU and triangular solves are launched inside the solve graph:
 * 1 = one kernel per elimination level (forward, with the LU step, then
 * backward), levels whose steps carry long gather lists as two kernels (the
 * level's pivots, one block each, then all its off-diagonal entries, one warp
 * each); 3 = as 1 but those levels as one kernel of one block per step (its
 * entries walked by that block); 2 = every level in one single-block kernel
 * with a barrier between levels (k_lu_fused: same per-step arithmetic, no
 * per-level launch); 0 = 2 up to 600 block rows (buses - 1) in the FP32-LU
 * form and 150 in FP64, else 1 (the default).  1 and 3 give the same factor.
 * Rebuilds the graph.  Not for metodo = denso. */
gbpf_status gbpf_solver_set_lu_launch(gbpf_solver *s, int mode);

/* The form gbpf_solve runs (gbpf_form).  gbpf_solver_create picks
 * GBPF_FORM_PERSISTENT for metodo = esparso in FP64 wherever the grid's state
 * fits one block's shared memory (up to ~1,900 buses) and GBPF_FORM_GRAPH
 * otherwise (the FP32-LU form may still be set to PERSISTENT); in FP64 the
 * same iterations, switch events, |V|, theta, history and flows come out of
 * both.  set: GBPF_E_UNSUPPORTED when the grid cannot run
 * PERSISTENT.  get: out[0] = the form, out[1] = kernel launches per solve of
 * it (for GRAPH: before the loop, per iteration and after; out[2] = per
 * iteration). */
gbpf_status gbpf_solver_set_form(gbpf_solver *s, int form);
gbpf_status gbpf_solver_get_form(const gbpf_solver *s, int out[3]);

/* The persistent form's LU plan: lu1 = 1 one-pass elimination levels (L kept
 * unscaled, so a level's entries need not wait for its pivots: one barrier a
 * level), 0 two-pass (pivots, then entries); narrow = 1 runs the levels
 * narrow enough for one warp on warp 0 alone with warp-level syncs; quad = 1
 * (FP64, one-pass levels) spreads each 2x2 block's four components over four
 * lanes, 0 keeps a block on one lane.  -1 keeps a knob (all -1: only
 * reports).  out[0..2] (may be NULL) = lu1, narrow, quad in force.  Plans
 * differ only in the order the LU sums its updates.  Rebuilds the persistent
 * graph; GBPF_E_UNSUPPORTED for a grid without that form. */
gbpf_status gbpf_solver_set_plan(gbpf_solver *s, int lu1, int narrow, int quad, int out[3]);

/* Solver facts: info[0..7] = nB, n blocks (nB-1), factor blocks (off-diagonal
 * per triangle), update pairs, forward levels, backward levels, graph nodes,
 * kernels launched per Newton iteration. */
gbpf_status gbpf_solver_info(const gbpf_solver *s, long long info[8]);

/* Device-resident timing hook: runs `repeats` solves from the stored start
 * with no host copies and returns the device time in ms (CUDA events on the
 * solver stream). */
gbpf_status gbpf_solver_time(gbpf_solver *s, int repeats, double *ms_total);

/* Wall ms of the set-up done by gbpf_solver_create: [0] Ybus (pattern on the
 * host, values on the device; calcYbusSp_eficinte), [1] device allocation,
 * [2] uploads of the grid and the factor structure (d_init* + cpyH2D of
 * GPU/main.cu:94-130), [3] symbolic analysis: ordering and factor structure
 * (Jstencil, GPU/limiteInjReat.cuh:220), [4] CUDA graph construction (the
 * library set-up of GPU/newtonRaphson.cuh:198-265). */
gbpf_status gbpf_solver_setup_times(const gbpf_solver *s, double ms[5]);

/* Per-phase device time (ms per pass, CUDA events on the solver stream, the
 * last solve's state left on the device, `repeats` passes after one warm-up):
 * [0] injections + limits + mismatch, [1] Jacobian fill, [2] LU
 * factorisation fused with forward substitution (all levels), [3] backward
 * substitution (all levels); with metodo = denso [1] the dense fill, [2] the
 * blocked LU, [3] the triangular solves.  bytes[] = algorithmic bytes of one
 * pass (in the factor's precision). */
gbpf_status gbpf_solver_profile(gbpf_solver *s, int repeats, double ms[4], long long bytes[4]);

/* ------------------------------------------------------------------------ */
/* Kernel-level entry points (each runs the product kernels on host inputs)  */
/* ------------------------------------------------------------------------ */

/* Device-assembled Ybus values in row-major CSR with sorted columns
 * (calcYbusSp_eficinte).  rowptr [nB+1], col/re/im [nnzY]. */
gbpf_status gbpf_ybus(gbpf_solver *s, int *rowptr, int *col, double *re, double *im);

/* P, Q injections at (V, theta) (calcPeficiente_0based / calcQeficiente_0based,
 * GPU/PQcalc.cuh:177-219). */
gbpf_status gbpf_eval_pq(gbpf_solver *s, const double *V, const double *theta, double *P,
                         double *Q);

/* Jacobian at (V, theta) for the limit flags limQ [nPV] (1 = PV bus held at a
 * Q limit, i.e. in barrasPQlim), returned as COO in the reference's row and
 * column numbering (Jstencil0based + SpCalcH/L/M/N).  *nnz = entries. */
gbpf_status gbpf_eval_jacobian(gbpf_solver *s, const double *V, const double *theta,
                               const int *limQ, int *row, int *col, double *val, int cap,
                               int *nnz);

/* Newton step: factorises the Jacobian at (V, theta, limQ) on the device and
 * solves J dx = g for g given in the reference's numbering (length
 * nB-1+nPQlim); replaces the cusolverSpDcsrlsvqr call of
 * GPU/newtonRaphson.cuh:455-478. */
gbpf_status gbpf_newton_step(gbpf_solver *s, const double *V, const double *theta,
                             const int *limQ, const double *g, double *dx);

/* ------------------------------------------------------------------------ */
/* Batched solves: many load scenarios of one or several topologies in one   */
/* persistent launch (no counterpart in the reference, which solves one grid */
/* per process run)                                                          */
/* ------------------------------------------------------------------------ */

typedef struct gbpf_batch gbpf_batch;

/* Topologies (symbolic analysis, device Ybus) for a batch.  Options used:
 * tolerancia, no_max_iter, lim_inj_reat, precision. */
gbpf_status gbpf_batch_create(const gbpf_grid *const *grids, int n_grids, const gbpf_options *o,
                              int device, gbpf_batch **out);
void gbpf_batch_free(gbpf_batch *b);

/* Instances: grid_of_inst[i] picks the topology of instance i; the bus arrays
 * are packed in instance order (instance i occupies nB of its grid entries)
 * and may be NULL (= the grid's own values).  Each given array is copied to
 * the device as it is (one transfer) and the inputs are packed there; the
 * caller may reuse the arrays on return.  Calling again with the same
 * grid_of_inst only replaces the inputs; a different list re-plans the
 * launch. */
gbpf_status gbpf_batch_set_instances(gbpf_batch *b, int n_inst, const int *grid_of_inst,
                                     const double *Pload, const double *Qload, const double *Pg,
                                     const double *Qg, const double *V0, const double *theta0);

/* Solves every instance: one graph launch (work-counter reset + one
 * persistent kernel, one thread block per instance at a time). */
gbpf_status gbpf_batch_solve(gbpf_batch *b);

/* The solve of gbpf_batch_solve without the wait: the graph is launched on
 * the batch's stream and the call returns.  gbpf_batch_wait waits for it.
 * Calls on one batch are ordered (set_instances and results wait for the
 * batch's earlier work); two batches in flight on their own streams let one
 * batch's bulk run beside the other's tail and its copies. */
gbpf_status gbpf_batch_launch(gbpf_batch *b);
gbpf_status gbpf_batch_wait(gbpf_batch *b);

/* `steps` solves spread round-robin over n batches, each on its own stream;
 * *ms = device ms from a common start event to the last batch's end (CUDA
 * events).  All batches on one device. */
gbpf_status gbpf_batch_time_pipelined(gbpf_batch *const *bs, int n, int steps, double *ms);

/* `repeats` batch solves back to back on the batch stream; device ms. */
gbpf_status gbpf_batch_time(gbpf_batch *b, int repeats, double *ms_total);

/* Device time of each kernel of the batch graph, averaged over `repeats`
 * launches (one synchronisation after each): ms[0] the block-per-instance
 * kernel, ms[1] the warp-per-instance kernel, ms[2] the hand-off launch that
 * resumes the warp kernel's long instances (CUDA events recorded inside the
 * graph, on the stream each kernel runs on).  0 for a kernel the batch does
 * not use. */
gbpf_status gbpf_batch_kernel_times(gbpf_batch *b, int repeats, double ms[3]);

/* Launch plan of the batch graph (no counterpart in the reference, which
 * solves one grid per process).  plan[0] warp mode: 1 = instances whose state
 * and factor fit a warp's slice of shared memory run one per warp, 0 = every
 * instance on a thread block of its own; plan[1] warps per block of the warp
 * kernel (default 8), 0 = as many as fit (at most 16); plan[2] the iteration at which an
 * instance still running leaves its warp for a thread block (0 = never);
 * plan[3] / plan[4] grouped lanes on levels with few pivots in those blocks /
 * in the warps (1 = on); plan[5] 1 = the thread-block kernel runs elimination
 * levels of at most 32 pivots and entries on one warp, without block
 * barriers between them; plan[6] / plan[7] 1 = the LU of the thread-block
 * kernel / of the warp kernel takes one pass per elimination level (L kept
 * unscaled, pivots and entries of a level side by side), 0 = two passes
 * (pivots, then entries scaled by the pivot inverse); plan[8] 1 = instances
 * on warps that start from their grid's own starting state (no V0 / theta0
 * given) take iteration 0 -- phasors, injections and the factored Jacobian,
 * which depend on the topology and the start only -- from one computation per
 * topology, and do only their own substitutions in it; plan[9] 1 = the
 * FP32-LU form updates its phasors by rotating them through the Newton step
 * instead of a sincos of every angle each iteration (0, the default, measured
 * faster on GB300); plan[10] the placement of thread-block instances'
 * state: level 1 keeps the per-bus arrays that no other bus's row reads
 * (theta, P, Q and, in the FP32-LU form, |V| and the FP64 phasor) in an
 * L2-resident global region instead of shared memory, level 2 every per-bus
 * array but the flags and the substitution vectors, level 3 is level 2
 * compiled for four blocks per SM (64 registers a thread); plan[10] = 1 takes
 * a level with at least 1.5x the instances per SM, else one with as many and
 * more factors in shared memory, else the lower level; 2, 3, 4 = level 1, 2,
 * 3 wherever it fits; 0 = level 0 (all in shared memory); plan[11] the same
 * for the warp kernel's instances (level 3 there: two blocks of 16 warps per
 * SM).  get_plan also returns plan[12]
 * warps per block in use, plan[13] instances on warps, plan[14] instances on
 * blocks, plan[15] / plan[16] the placement level in use for blocks / warps
 * (plan[17..19] = 0).  Setting a plan rebuilds the batch graph. */
gbpf_status gbpf_batch_get_plan(const gbpf_batch *b, int plan[20]);
gbpf_status gbpf_batch_set_plan(gbpf_batch *b, const int plan[12]);

/* Autotuner: a coordinate search over plan[0..11] on the current instances,
 * from the default plan.  Each knob takes each of its values in turn with the
 * others fixed; a value is kept when the whole batch solve (best of `repeats`
 * timed graph launches after one warm-up, CUDA events on the batch stream) is
 * at least 2 % faster; a second sweep runs when the first changed the plan,
 * then joint trials of the warp kernel's placement level 3 with 9, 10 and 12
 * warps per block (each change alone is slower).  The best plan stays set; plan receives it (as gbpf_batch_get_plan) and
 * ms[0] / ms[1] the batch time of the default and of the chosen plan.  The
 * trial solves overwrite the instances' results. */
gbpf_status gbpf_batch_autotune(gbpf_batch *b, int repeats, int plan[20], float ms[2]);

/* Per-instance results of the last batch solve (any pointer may be NULL);
 * V/theta/P/Q packed like the inputs.  Each array is copied from the device
 * straight into the caller's memory (one transfer, no staging copy). */
gbpf_status gbpf_batch_results(gbpf_batch *b, int *iterations, int *status, double *final_mismatch,
                               int *n_events, double *V, double *theta, double *Pcalc, double *Qcalc);

/* Switch events of one instance (first 16 kept), 4 ints each as in
 * gbpf_solver_events. */
gbpf_status gbpf_batch_events(gbpf_batch *b, int inst, int *ev, int cap, int *n);

/* Switch events of every instance in one call: ev[(i * cap + k) * 4 ..] holds
 * event k of instance i (cap <= 16, sorted as gbpf_batch_events sorts them,
 * unused slots zero) and n[i] the events instance i recorded (it may exceed
 * cap, which then keeps the first cap).  The bulk form of gbpf_batch_events,
 * for comparing the switch paths of two precisions scenario by scenario
 * (the reference prints them per solve, GPU/limiteInjReat.cuh:12-34). */
gbpf_status gbpf_batch_events_all(gbpf_batch *b, int *ev, int cap, int *n);

/* For callers that cannot allocate device memory when they solve.  No
 * counterpart in the reference.  cudaMalloc can synchronise the device and
 * takes an unbounded time, so a caller with a fixed cycle time (a real-time
 * contingency loop, a control-room state estimator) forbids it after
 * start-up; other callers run inside a host framework whose device memory
 * belongs to its own allocator.  Solves n_inst instances like
 * gbpf_batch_set_instances + gbpf_batch_solve, on caller-owned DEVICE buffers
 * packed in instance order (V0, theta0, Pliq, Qliq, Qload in; V, theta, Pcalc,
 * Qcalc, iterations, status, final_mismatch out); grid_of_inst is a HOST
 * array, read before the call returns.  Allocates nothing: all scratch lives
 * in one static 8 MiB device array, each GPU that loads the library holds it
 * until exit, and every call shares it, so calls that overlap on the GPU race.
 * gbpf_batch_create does the one-time set-up for its device (the array's
 * device address).  Rejects with GBPF_E_ARG an instance count or a factor that
 * does not fit the scratch, and a grid whose state does not fit one block's
 * shared memory.  Does not record switch events.  The solve is asynchronous
 * on `stream` (a cudaStream_t; NULL = the batch's stream). */
gbpf_status gbpf_batch_solve_noalloc(gbpf_batch *b, int n_inst, const int *grid_of_inst,
                                     const double *V0, const double *theta0, const double *Pliq,
                                     const double *Qliq, const double *Qload, double *V,
                                     double *theta, double *Pcalc, double *Qcalc, int *iterations,
                                     int *status, double *final_mismatch, void *stream);

/* ------------------------------------------------------------------------ */
/* Learned warm start (no counterpart in the reference, whose Newton loop    */
/* always starts from v_inicial / theta_inicial, GPU/sistInfo.h:62-242)      */
/* ------------------------------------------------------------------------ */

/* A dense network features -> n_hidden_layers x n_hidden_width (GELU) ->
 * outputs, bf16 weights with fp32 master copies, trained with Adam on the GPU
 * by the library's own tensor-core (tcgen05) kernels.  linear_skip != 0 adds
 * a linear path from the features to the outputs (y = MLP(x) + S x), summed
 * in the output layer's accumulator; it lets the network represent the
 * near-linear, full-rank response of the bus angles to the injections, which
 * a hidden width below the bus count cannot.  Layer index n_hidden_layers + 1
 * of gbpf_mlp_params is S (no bias).  For a warm start of a grid with nB
 * buses: n_in = 3*nB with features [Pliq | Qliq | V0] of every bus (p.u.,
 * file bus order), or n_in = 2*nB with [Pliq | Qliq] where the scenarios'
 * starting voltages do not vary (constant features normalise to zeros, which
 * the network would multiply for nothing), and n_out = 2*nB with outputs
 * [|V| | theta]. */
typedef struct gbpf_mlp gbpf_mlp;
gbpf_status gbpf_mlp_create(int n_in, int n_hidden_width, int n_hidden_layers, int n_out, int linear_skip,
                            unsigned long long seed, int device, gbpf_mlp **out);
void gbpf_mlp_free(gbpf_mlp *m);
/* dims = n_in, hidden width, hidden layers, n_out, linear_skip. */
gbpf_status gbpf_mlp_dims(const gbpf_mlp *m, int dims[5]);

/* Training set: X [n, n_in] and Y [n, n_out] (host, row-major, raw units).
 * Sets the per-feature normalisation (mean, 1/std of inputs; mean, std of
 * outputs) from the data and keeps a normalised copy on the device. */
gbpf_status gbpf_mlp_set_data(gbpf_mlp *m, const float *X, const float *Y, int n);

/* `epochs` passes over the training set in shuffled mini-batches of `batch`
 * rows (a multiple of 8; the last partial batch of each epoch is dropped),
 * mean-squared error on the normalised outputs, Adam (beta 0.9 / 0.999,
 * eps 1e-8) at a learning rate that falls from lr to lr_final along a cosine
 * over the steps of this call (lr_final == lr: constant).  epoch_loss[e] (may
 * be NULL) = mean loss of epoch e; *ms_total (may be NULL) = device time of
 * all epochs. */
gbpf_status gbpf_mlp_train(gbpf_mlp *m, int epochs, int batch, float lr, float lr_final,
                           unsigned long long seed, float *epoch_loss, double *ms_total);

/* Training loss over the normalised output residual e (one row per sample):
 * (|e A|^2 + lam |e|^2) / (rows * n_out) with A [n_out, k] (host, row-major,
 * rounded to bf16 on the device; the loss stays a sum of squares); A = NULL
 * restores the mean squared error (lam ignored).  For a warm start, A = S J0^T
 * with J0 the Newton Jacobian at a typical solution and S the output scales
 * makes |e A| the linearised mismatch of the predicted start, which is what
 * decides how many Newton iterations the start saves. */
gbpf_status gbpf_mlp_set_loss_metric(gbpf_mlp *m, const float *A, int k, float lam);

/* Limit of the operand-ring mbarrier waits of the network's tensor-core GEMMs,
 * in SM clock cycles (0 = the default, about 2 s at 2 GHz; no counterpart in
 * the reference, which has no network).  A wait that runs out makes the GEMM
 * stop issuing work, wait for its tensor-core operations and copies already in
 * flight (fixed ~2 s bound), free its tensor memory and return; the call then
 * returns GBPF_E_TIMEOUT and the handle stays usable.  Applies to GEMMs
 * launched afterwards by gbpf_mlp_predict, gbpf_mlp_gradients and the
 * warm-started solves; the training graph keeps the limit in force when
 * gbpf_mlp_train first builds it. */
gbpf_status gbpf_mlp_set_wait_limit(gbpf_mlp *m, long long cycles);

/* Y [n, n_out] = network(X [n, n_in]), raw units in and out. */
gbpf_status gbpf_mlp_predict(gbpf_mlp *m, const float *X, int n, float *Y);

/* Loss and gradients of one batch of NORMALISED rows Xn [n, n_in], Yn
 * [n, n_out] (n a multiple of 8) at the current parameters, without an
 * update: dW = the weight gradients of every layer concatenated (layer l is
 * [out_l, in_l] row-major; the skip S last, [n_out, n_in]), db = the bias
 * gradients concatenated. */
gbpf_status gbpf_mlp_gradients(gbpf_mlp *m, const float *Xn, const float *Yn, int n, float *loss,
                               float *dW, float *db);

/* Parameters of layer `layer` (0 = first): W [out, in] row-major, b [out]. */
gbpf_status gbpf_mlp_params(gbpf_mlp *m, int layer, float *W, float *b);
gbpf_status gbpf_mlp_set_params(gbpf_mlp *m, int layer, const float *W, const float *b);
/* Normalisation: x_norm = (x - in_mean) * in_scale; y = y_norm * out_scale + out_mean. */
gbpf_status gbpf_mlp_norm(const gbpf_mlp *m, float *in_mean, float *in_scale, float *out_mean,
                          float *out_scale);
gbpf_status gbpf_mlp_set_norm(gbpf_mlp *m, const float *in_mean, const float *in_scale,
                              const float *out_mean, const float *out_scale);

/* Batched Newton from the network's start: the current instances (all on one
 * grid of nB buses; network n_in = 3*nB or 2*nB, n_out = 2*nB) are turned into
 * features on the device, the network predicts |V| (PQ buses) and theta
 * (non-slack buses), and each instance starts from the prediction when its
 * initial mismatch is smaller than that of the instance's own start
 * (V0/theta0 of gbpf_batch_set_instances, by default the flat start), else
 * from its own start.  Instances whose predicted start does not converge are
 * solved again from their own start, in the same launch.  Iteration 0 of a
 * predicted run is a chord step: its Newton system is solved with the factor
 * of the Jacobian at the network's mean output (out_mean, with the grid's PV
 * set points and slack angle), factored once per network and grid, instead
 * of the instance's own Jacobian; later iterations are full Newton steps.
 * Instances are served in order of falling predicted angle spread (max - min
 * theta of the prediction), the most stressed scenarios first.  Results as for
 * gbpf_batch_solve (gbpf_batch_results); an instance on its own start gets
 * no_max_iter iterations.  start_kind[i] (may be NULL): 0 own start chosen up
 * front, 1 predicted start converged, 2 predicted start failed (no
 * convergence within min(no_max_iter, 10) iterations, or a solution whose
 * |V| lies more than 0.05 p.u. from the prediction) and was replaced;
 * warm_iterations[i] (may be NULL): iterations of the predicted-start
 * attempt (0 when not attempted); *ms (may be NULL): device time of the whole
 * sequence, network inference included. */
gbpf_status gbpf_batch_solve_warm(gbpf_batch *b, gbpf_mlp *m, int *start_kind, int *warm_iterations,
                                  double *ms);

/* Order two batches' warm-started solves on the device: the next solve
 * enqueued with gbpf_batch_solve_warm_launch on b starts when prev's last
 * warm-started solve (its result copies included) has ended, while the host
 * goes on enqueueing.  For keeping two batches in flight without their Newton
 * launches sharing the GPU's L2 (no counterpart in the reference). */
gbpf_status gbpf_batch_follow(gbpf_batch *b, const gbpf_batch *prev);

/* gbpf_batch_solve_warm in two halves: _launch enqueues every step on the
 * batch's stream and returns; _wait waits for it and fills start_kind,
 * warm_iterations and *ms as gbpf_batch_solve_warm does.  Between the two the
 * caller may work with other batches (each batch has its own stream and its
 * own workspace for the network, so batches that share a network can have
 * warm-started solves in flight at once); gbpf_batch_set_instances on this
 * batch is refused until the wait. */
gbpf_status gbpf_batch_solve_warm_launch(gbpf_batch *b, gbpf_mlp *m);
gbpf_status gbpf_batch_solve_warm_wait(gbpf_batch *b, int *start_kind, int *warm_iterations, double *ms);

/* Device ms of `steps` warm-started solves spread round-robin over n batches
 * (all on one device, none with a warm-started solve in flight), each on its
 * own stream; a batch is waited for before it is launched again, and each
 * solve starts on the device after the previous one has ended (as
 * gbpf_batch_follow), so the host enqueues ahead without two Newton launches
 * sharing the L2.  From a start event every stream waits for to the latest
 * stream's end. */
gbpf_status gbpf_batch_time_warm_pipelined(gbpf_batch *const *bs, int n, gbpf_mlp *m, int steps, double *ms);

/* Device time of the last gbpf_batch_solve_warm by phase: ms[0] the network
 * (features and inference), ms[1] the start choice and the queue order, ms[2]
 * the Newton launch (restarts included).  Zeros before the first call. */
gbpf_status gbpf_batch_warm_phases(const gbpf_batch *b, double ms[3]);

/* info[0..7] = topologies, instances, packed buses, resident thread blocks,
 * dynamic shared memory per block of the block-per-instance kernel,
 * topologies whose factor is in shared memory, global scratch bytes per
 * block, instances served by the warp-per-instance kernel. */
gbpf_status gbpf_batch_info(const gbpf_batch *b, long long info[8]);

/* Device query for the driver's banner (initGPU, GPU/sistema.cuh:426-468):
 * *count = CUDA devices; name of `device`; props = major, minor, warp size,
 * max threads per SM, max threads per block, SM count. */
gbpf_status gbpf_device_info(int device, int *count, char *name, size_t name_cap, int props[6]);

/* Text of the last error on this thread. */
const char *gbpf_last_error(void);
const char *gbpf_status_str(gbpf_status st);

#ifdef __cplusplus
}
#endif
#endif /* GBPF_H */
