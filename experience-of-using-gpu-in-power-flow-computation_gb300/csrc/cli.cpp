// cli.cpp -- `gbpf`, the command-line driver: the process-level drop-in for the
// reference's GPU executable (GPU/main.cu:25-216).  Reads data.txt (or the path
// given as the first argument), reads arq_entrada, solves on the GPU and prints
// what the reference prints: the option echo, the method banner, the GPU
// banner, the reactive-limit lines and max(g) trace, and the per-bus table of
// impressao2 (GPU/impressao.h:47-80), then the execution report on screen
// (benchmarksPrint, GPU/impressao.h:125-337) and the benchmark CSV row
// (benchmarksPrintFile, GPU/impressao.h:339-558).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "gbpf.h"

static const char *EVENT_TEXT[6] = {
    "", "PV -> PQ (limite superior)", "PQ (limite inferior) -> PQ (limite superior)",
    "PV -> PQ (limite inferior)", "PQ (limite superior) -> PQ (limite inferior)", "PQ -> PV"};

// Times of one run in the reference's benchmark categories (ms).  Set-up
// phases are wall times measured by the library; the Newton phases are the
// device time of one pass of each phase (gbpf_solver_profile) -- the Newton
// loop runs as one CUDA graph, so there is no host-side timer per iteration.
struct RunTimes {
    double total = 0, ybus = 0, alloc = 0, upload = 0, lib = 0, stencil = 0;
    double pq_pass = 0, jac_pass = 0, lin_pass = 0, processo = 0, fluxo = 0;
    int iters = 0, pq_passes = 0;
};

static std::string met2str(const gbpf_options &o) {  // GPU/impressao.h:82-101, hibridoC of :342-347
    switch (o.metodo) {
    case GBPF_METODO_DENSO: return "denso";
    case GBPF_METODO_ESPARSO: return "esparso";
    case GBPF_METODO_HIBRIDOA: return "hibridoA";
    case GBPF_METODO_HIBRIDOB: return "hibridoB";
    case GBPF_METODO_HIBRIDOC: return "hibridoC";
    default: return "nda";
    }
}

// printDoubleToFile (GPU/impressao.h:119-123): "%f" with a decimal comma, then ';'
static std::string csv_num(double x) {
    char b[64];
    std::snprintf(b, sizeof b, "%f", x);
    std::string s(b);
    const size_t p = s.find('.');
    if (p != std::string::npos) s[p] = ',';
    return s + ";";
}

// The benchmark CSV row of benchmarksPrintFile: file out_<double|float>_<metodo>-<input
// without extension>.csv, created with the reference's two header lines (byte
// for byte, including the replacement characters its source file carries),
// one row appended per run, numbered by the lines already in the file.
static void write_csv(const gbpf_options &o, const RunTimes &t) {
    std::string in = o.arq_entrada;
    const size_t dot = in.find_last_of('.');
    const std::string name = std::string("out_") + (o.precision == GBPF_PREC_FP32_IR ? "float_" : "double_") +
                             met2str(o) + "-" + in.substr(0, dot) + ".csv";
    unsigned n = 1;
    {
        std::ifstream f(name, std::ios::binary);
        if (f.good()) {
            unsigned lines = 0;
            char c;
            while (f.get(c)) lines += c == '\n';
            n = lines - 1;
        } else {
            std::ofstream h(name, std::ios::binary);
            h << "Execucao;Aviso;ms total;no iteracoes;ms Ybus;ms Init GPU;;;ms Inicializacao;ms calcPQ;;"
                 "ms Jacobiano;;ms Sistema Linear;;ms Processo;ms Fluxo;\n;;;;;total; Aloca\xEF\xBF\xBD\xEF\xBF\xBDo "
                 "Vari\xEF\xBF\xBDveis iniciais; Aloca\xEF\xBF\xBD\xEF\xBF\xBDo de vari\xEF\xBF\xBDveis esparsas; "
                 "Biblioteca; total; medio por iteracao; total; medio por iteracao; total; medio por iteracao; "
                 "Iterativo;\n";
        }
    }
    const double it = (double)t.iters;
    const bool dense = o.metodo == GBPF_METODO_DENSO;
    std::string row = std::to_string(n) + ";" + ";" + csv_num(t.total) + std::to_string(t.iters) + ";";
    row += csv_num(t.ybus) + csv_num(t.alloc + t.upload) + csv_num(t.alloc) + csv_num(t.upload) + csv_num(t.lib);
    row += csv_num(t.pq_pass * t.pq_passes) + csv_num(t.pq_pass * t.pq_passes / it);
    const double jac = t.jac_pass * t.iters + (dense ? 0.0 : t.stencil);
    row += csv_num(jac) + csv_num(jac / it);
    row += csv_num(t.lin_pass * t.iters) + csv_num(t.lin_pass * t.iters / it);
    row += csv_num(t.processo) + csv_num(t.fluxo) + "\n";
    std::ofstream f(name, std::ios::binary | std::ios::app);
    f << row;
}

// The execution report of benchmarksPrint (BENCHMARK_MODE on).
static void print_report(const gbpf_options &o, const RunTimes &t) {
    const bool dense = o.metodo == GBPF_METODO_DENSO;
    std::printf("\n Relatorio de execucao:\n\n");
    std::printf("*Geral***********************************\n\n ");
    std::printf(" Tempo total de execucao: %f ms.\n Numero de iteracoes: %d.\n\n", t.total, t.iters);
    std::printf("*Ybus************************************\n\n");
    std::printf(" Tempo total: %f ms.\n\n", t.ybus);
    std::printf("*Init GPU********************************\n\n");
    std::printf(" acao                        -  tempo de execucao\n");
    std::printf(" alocacao de memoria inicial - %14f ms (alem do inicio da comunicacao com a GPU)\n", t.alloc);
    std::printf(" alocacao de varia. esparsas - %14f ms\n", t.upload);
    std::printf("-----------------------------\n");
    std::printf(" Tempo total: %f ms.\n\n", t.alloc + t.upload);
    std::printf("*Inicializacao das Bibliotecas***********\n\n");
    std::printf(" Tempo total: %f ms.\n\n", t.lib);
    std::printf("*CalcPQ**********************************\n\n");
    std::printf("*Tempo nao inclui transferencias de dados para o host!\n\n");
    std::printf(" iteracao - tempo de execucao\n");
    for (int i = 0; i < t.pq_passes; i++) std::printf(" %8d - %14f ms\n", i, t.pq_pass);
    std::printf("-----------------------------\n");
    std::printf(" Tempo total: %f ms.\n", t.pq_pass * t.pq_passes);
    std::printf(" Tempo medio: %f ms.\n\n", t.pq_pass * t.pq_passes / (double)t.iters);
    if (dense) {
        std::printf("*Jacobiano*******************************\n\n");
        std::printf(" iteracao - tempo de execucao\n");
        for (int i = 0; i < t.iters; i++) std::printf(" %8d - %14f ms\n", i, t.jac_pass);
        std::printf("-----------------------------\n");
        std::printf(" Tempo total: %f ms.\n", t.jac_pass * t.iters);
        std::printf(" Tempo medio: %f ms.\n\n", t.jac_pass * t.iters / (double)t.iters);
    } else {
        const double tot = t.stencil + t.jac_pass * t.iters;
        std::printf("*Jacobiano Stencil***********************\n");
        std::printf("  acao  - iteracao - tempo de execucao\n");
        std::printf(" constr - %8d - %14f ms\n", 0, t.stencil);
        for (int i = 0; i < t.iters; i++) std::printf(" preenc - %8d - %14f ms\n", i, t.jac_pass);
        std::printf("-----------------------------\n");
        std::printf(" Tempo total: %f ms.\n", tot);
        std::printf(" Tempo medio: %f ms (por iteracao).\n\n", tot / (double)t.iters);
    }
    std::printf("*Sistema Linear**************************\n\n");
    std::printf(" iteracao - tempo de execucao\n");
    for (int i = 0; i < t.iters; i++) std::printf(" %8d - %14f ms\n", i, t.lin_pass);
    std::printf("-----------------------------\n");
    std::printf(" Tempo total: %f ms.\n", t.lin_pass * t.iters);
    std::printf(" Tempo medio: %f ms.\n\n", t.lin_pass * t.iters / (double)t.iters);
    std::printf("*Processo Iterativo**********************\n\n");
    std::printf(" Tempo total: %f ms.\n\n", t.processo);
    std::printf("*Fluxo***********************************\n\n");
    std::printf(" Tempo total: %f ms.\n\n", t.fluxo);
    std::printf("*****************************************\n");
}

// showVec (GPU/dim.h:11-37): '[' before the first value, one value a line, a
// space before the others and ']' after the last, fixed with prec decimals.
// An empty vector prints "[]" (the reference reads outside the array there).
static void show_vec(const double *v, int n, int prec) {
    if (n <= 0) { std::printf("[]\n"); return; }
    std::printf("[%.*f\n", prec, v[0]);
    for (int i = 1; i < n - 1; i++) std::printf(" %.*f\n", prec, v[i]);
    std::printf(" %.*f]\n", prec, v[n - 1]);
}
static void show_vec(const int *v, int n) {
    if (n <= 0) { std::printf("[]\n"); return; }
    std::printf("[%d\n", v[0]);
    for (int i = 1; i < n - 1; i++) std::printf(" %d\n", v[i]);
    std::printf(" %d]\n", v[n - 1]);
}

static void print_events(const int *ev, int n) {  // chkLimQ, GPU/limiteInjReat.cuh:6-34
    std::printf("\n");
    for (int e = 0; e < n; e++)
        std::printf("Barra %d [%d]: %s\n", ev[4 * e + 1], ev[4 * e + 2], EVENT_TEXT[ev[4 * e + 3]]);
}

// verbose_mode = ON: the dumps of mNR printed from gbpf_solve_traced's records,
// in the reference's order (GPU/newtonRaphson.cuh:270-563, GPU/Jacobiano.cuh:
// 216-220 and 382-410, GPU/PQcalc.cuh:304-320 and 417-432 for denso).
struct Verbose {
    const gbpf_options *o = nullptr;
    std::vector<double> Qmin, Qmax;
    std::vector<double> prevJ;  // the Jacobian value array as the last fill left it
    bool started = false;
};

static void verbose_trace(const gbpf_trace *t, void *user) {
    Verbose &vb = *(Verbose *)user;
    const gbpf_options &o = *vb.o;
    const int it = t->iteration, nB = t->nB;
    const bool dense = o.metodo == GBPF_METODO_DENSO;
    switch (t->stage) {
    case GBPF_TRACE_EVAL: {
        if (it >= o.no_max_iter) return;  // the loop has ended before this evaluation
        if (!vb.started) {
            vb.started = true;
            if (o.lim_inj_reat) {  // printAlLim after initLim, GPU/limiteInjReat.cuh:226-242
                std::printf("nPQlim = %d\nnPVlim = %d\n", t->nPQlim, t->nPVlim);
                std::printf("limQ:\n");
                show_vec(t->limQ, t->nPV);
                std::printf("barrasPVlim:\n");
                show_vec(t->pv_lim, t->nPVlim);
                std::printf("barrasPQlim:\n");
                show_vec(t->pq_lim, t->nPQlim);
                std::printf("limQinf:\n");
                show_vec(vb.Qmin.data(), t->nPV, 4);
                std::printf("limQsup:\n");
                show_vec(vb.Qmax.data(), t->nPV, 4);
                std::printf("QliqLim:\n");
                show_vec(t->QliqLim, nB, 4);
            }
        }
        std::printf("\n****************************************************************** ITERACAO %d "
                    "******************************************************************\n", it);
        if (dense) {  // d_dnCalcPf_sha / d_dnCalcQf_sha print every bus
            for (int k = 1; k <= nB; k++) std::printf("P_%d\t= %f\n", k, t->P[k - 1]);
            for (int k = 1; k <= nB; k++) std::printf("Q_%d\t= %f\n", k, t->Q[k - 1]);
        }
        if (t->limit_check) {
            print_events(t->events, t->n_events);
            vb.prevJ.clear();  // a new stencil, its values zeroed (GPU/limiteInjReat.cuh:149-150)
        }
        std::printf("Pcalc^(%d) =\n", it);
        show_vec(t->P, nB, 4);
        std::printf("\nQcalc^(%d) =\n", it);
        show_vec(t->Q, nB, 4);
        std::printf("\ndeltaP^(%d) =\n", it);
        show_vec(t->g, nB - 1, 4);
        std::printf("\ndeltaQ^(%d) =\n", it);
        show_vec(t->g + nB - 1, t->nPQlim, 4);
        std::printf("\nlimQ:\n");
        show_vec(t->limQ, t->nPV);
        std::printf("\nbarrasPVlim:\n");
        show_vec(t->pv_lim, t->nPVlim);
        std::printf("\nbarrasPQlim:\n");
        show_vec(t->pq_lim, t->nPQlim);
        std::printf("\nlimQinf:\n");
        show_vec(vb.Qmin.data(), t->nPV, 4);
        std::printf("\nlimQsup:\n");
        show_vec(vb.Qmax.data(), t->nPV, 4);
        std::printf("\nQliqLim:\n");
        show_vec(t->QliqLim, nB, 4);
        std::printf("\nmax(g) = %e", t->max_g);
        if (t->converged) std::printf("\n\nbreak!\nmax(g) = %e\n\n", t->max_g);
        else if (!t->done) std::printf("     ...     continua:\n\n");
        break;
    }
    case GBPF_TRACE_JACOBIAN: {
        const int nnz = t->nnzJ, dim = t->n_g;
        if (dense) {  // calcJacLim's JacobianoN, showMat (GPU/dim.h:157-167)
            std::vector<double> A((size_t)dim * dim, 0.0);
            for (int e = 0; e < nnz; e++) A[(size_t)t->jrow[e] * dim + t->jcol[e]] = t->jval[e];
            std::printf("JacobianoN =\n\n[");
            for (int r = 0; r < dim; r++) {
                for (int c = 0; c < dim; c++) std::printf("%5.1f ", A[(size_t)r * dim + c]);
                std::printf("\n ");
            }
            std::printf("]\n\n");
        } else {
            // SpCalcJac fills H, L, M, N in turn and prints the value array
            // after the first three; entries not yet filled hold the last fill's
            // values, or zero on a new stencil (GPU/limiteInjReat.cuh:86-87)
            std::vector<double> cur(vb.prevJ.size() == (size_t)nnz ? vb.prevJ : std::vector<double>(nnz, 0.0));
            const int np = nB - 1;
            const char *name[3] = {"H", "L", "M"};
            for (int part = 0; part < 3; part++) {
                for (int e = 0; e < nnz; e++) {
                    const bool prow = t->jrow[e] < np, pcol = t->jcol[e] < np;
                    const bool in = part == 0 ? (prow && pcol) : part == 1 ? (!prow && !pcol) : (!prow && pcol);
                    if (in) cur[e] = t->jval[e];
                }
                std::printf("%s^(%d) =\n", name[part], it);
                show_vec(cur.data(), nnz, 5);
            }
            std::printf("J^(%d) =\n", it);
            show_vec(t->jval, nnz, 5);
            vb.prevJ.assign(t->jval, t->jval + nnz);
        }
        std::printf("V^(%d) = \n", it);
        show_vec(t->V, nB, 5);
        std::printf("theta^(%d) = \n", it);
        show_vec(t->theta, nB, 5);
        std::printf("deltaPQ = \n");
        show_vec(t->g, t->n_g, 5);
        break;
    }
    case GBPF_TRACE_STEP:
        std::printf("\n (deltaX)g^(%d) = \n", it);
        show_vec(t->g, t->n_g, 5);
        break;
    case GBPF_TRACE_UPDATE:
        std::printf("V^(%d) = \n", it);
        show_vec(t->V, nB, 6);
        std::printf("theta^(%d) = \n", it);
        show_vec(t->theta, nB, 6);
        break;
    default: break;
    }
}

static int fail(const char *what, gbpf_status st) {
    std::fprintf(stderr, "gbpf: %s: %s (%s)\n", what, gbpf_status_str(st), gbpf_last_error());
    return 1;
}

int main(int argc, char **argv) {
    const char *data = argc > 1 ? argv[1] : "data.txt";
    gbpf_options o;
    gbpf_options_default(&o);
    static char echo[1 << 16];
    if (gbpf_options_load(data, &o, echo, sizeof echo) != GBPF_OK) {
        std::printf("ERRO: A ABERTURA DO ARQUIVO FALHOU!");  // GPU/sistInfo.h:72
        return 1;
    }
    std::fputs(echo, stdout);

    gbpf_grid *g = nullptr;
    static char msg[1 << 20];
    gbpf_status st = gbpf_grid_read(o.arq_entrada, o.v_inicial, o.theta_inicial, &g, msg, sizeof msg);
    if (st != GBPF_OK) {
        std::printf("Erro ao abrir o arquivo...");  // GPU/arquivo.h:266
        return fail("reading input", st);
    }
    // reader notices, in file order (GPU/sistema.h:596-611)
    for (char *line = std::strtok(msg, "\n"); line; line = std::strtok(nullptr, "\n")) {
        if (!std::strncmp(line, "Ramo ", 5)) {
            if (!o.laconic_mode) std::printf("\n%s", line);
        } else {
            std::printf("\n%s\n", line);
        }
    }

    const char *banner = nullptr;
    switch (o.metodo) {  // GPU/main.cu:35-60
    case GBPF_METODO_DENSO: banner = "[DENSO]"; break;
    case GBPF_METODO_HIBRIDOA: banner = "[HIBRIDO A]"; break;
    case GBPF_METODO_HIBRIDOB: banner = "[HIBRIDO B]"; break;
    case GBPF_METODO_HIBRIDOC: banner = "[HIBRIDO C]"; break;
    case GBPF_METODO_ESPARSO: banner = "[ESPARSO]"; break;
    default: break;
    }
    if (banner) std::printf(o.laconic_mode ? "%s\n\n" : "\n\n%s\n\n", banner);
    else std::printf("[METODO] METODO INVALIDO LIDO DO ARQUIVO!\n\n");
    if (o.metodo != GBPF_METODO_ESPARSO && o.metodo != GBPF_METODO_DENSO && o.metodo != GBPF_METODO_NDA)
        std::fprintf(stderr, "gbpf: metodo %s runs the GPU sparse solve (no host library solve)\n",
                     banner ? banner : "?");

    // GPU banner of initGPU (GPU/sistema.cuh:426-468)
    int count = 0, props[6] = {0};
    char name[256] = {0};
    st = gbpf_device_info(0, &count, name, sizeof name, props);
    if (st != GBPF_OK && st != GBPF_E_ARG) return fail("device query", st);
    std::printf("\n\n");
    if (count == 0) {
        std::printf("There are no available device(s) that support CUDA\n");
        return 1;
    }
    std::printf("Detected %d CUDA Capable device(s)\n", count);
    if (!o.laconic_mode) {
        std::printf("GPU Device %d: \"%s\" with compute capability %d.%d\n\n", 0, name, props[0], props[1]);
        std::printf("  Warp size:                                    %d\n", props[2]);
        std::printf("  Maximum number of threads per multiprocessor: %d\n", props[3]);
        std::printf("  Maximum number of threads per block:          %d\n", props[4]);
        std::printf("  (%2d) Multiprocessors, (%3d) CUDA Cores/MP:     %d CUDA Cores\n", props[5], 128,
                    128 * props[5]);
    }

    using clk = std::chrono::steady_clock;
    auto ms_since = [](clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); };
    RunTimes tm;
    const auto t_start = clk::now();
    gbpf_solver *s = nullptr;
    st = gbpf_solver_create(g, &o, 0, &s);
    if (st != GBPF_OK) return fail("solver setup", st);
    gbpf_result r{};
    Verbose vb;
    auto t0 = clk::now();
    if (o.verbose_mode) {
        int dims[8];
        gbpf_grid_dims(g, dims);
        vb.o = &o;
        vb.Qmin.resize(dims[2] + 1);
        vb.Qmax.resize(dims[2] + 1);
        gbpf_grid_pvpq(g, nullptr, vb.Qmin.data(), vb.Qmax.data(), nullptr, nullptr);
        st = gbpf_solve_traced(s, &r, verbose_trace, &vb);
    } else {
        st = gbpf_solve(s, &r);
    }
    tm.processo = ms_since(t0);
    if (st != GBPF_OK && st != GBPF_E_NOCONV) return fail("solve", st);
    {
        int dims[8];
        gbpf_grid_dims(g, dims);
        std::vector<double> a(dims[0]), b(dims[0]), c(dims[0]), d(dims[0]), f(4 * (size_t)dims[1] + 4);
        gbpf_solver_state(s, a.data(), b.data(), c.data(), d.data());
        t0 = clk::now();
        gbpf_solver_flows(s, f.data(), f.data() + dims[1], f.data() + 2 * dims[1], f.data() + 3 * dims[1]);
        tm.fluxo = ms_since(t0);
    }
    tm.total = ms_since(t_start);
    tm.iters = r.iterations;
    tm.pq_passes = r.converged ? r.iterations + 1 : r.iterations;

    // trace of mNR in iteration order: limit lines (GPU/limiteInjReat.cuh:6-34)
    // and max(g) (GPU/newtonRaphson.cuh:418-420)
    const int cap = o.no_max_iter + 2;
    std::vector<double> hist(cap);
    std::vector<int> trig(cap), ev(4 * 4096);
    int nh = 0, nt = 0, ne = 0;
    gbpf_solver_history(s, hist.data(), cap, &nh);
    gbpf_solver_triggers(s, trig.data(), cap, &nt);
    gbpf_solver_events(s, ev.data(), 4096, &ne);
    const int last = r.converged ? r.iterations : std::min(r.iterations, o.no_max_iter) - 1;
    int e = 0;
    for (int it = 0; it <= last && it < nh && !o.verbose_mode; it++) {  // verbose: printed as it ran
        if (it < nt && trig[it]) {
            int e1 = e;
            while (e1 < ne && ev[4 * e1] == it) e1++;
            print_events(ev.data() + 4 * e, e1 - e);
            e = e1;
        }
        if (o.output_iter && !o.laconic_mode) std::printf("\nmax(g) = %e", hist[it]);
    }

    if (!o.laconic_mode && o.output_ans) {  // impressao2, GPU/impressao.h:47-80
        int dims[8];
        gbpf_grid_dims(g, dims);
        const int nB = dims[0], nL = dims[1];
        std::vector<int> id(nB), de(nL), pa(nL);
        std::vector<double> V(nB), th(nB), P(nB), Q(nB), Pl(nB), Ql(nB);
        std::vector<double> Pdp(nL), Ppd(nL), Qdp(nL), Qpd(nL);
        gbpf_grid_buses(g, id.data(), nullptr, nullptr, nullptr, Pl.data(), Ql.data(), nullptr, nullptr,
                        nullptr, nullptr);
        gbpf_grid_branches(g, de.data(), pa.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
        gbpf_solver_state(s, V.data(), th.data(), P.data(), Q.data());
        gbpf_solver_flows(s, Pdp.data(), Ppd.data(), Qdp.data(), Qpd.data());
        std::printf("\n\n                                 FLUXOS DE POTENCIA\n");
        std::printf("        BUS      V         ANG        Pli        Qli        Pge        Qge      TO        PIJ          QIJ\n");
        for (int i = 0; i < nB; i++) {
            std::printf("      %4d%11.5f%11.5f%11.5f%11.5f%11.5f%11.5f  ", id[i], V[i], th[i], P[i], Q[i],
                        P[i] + Pl[i], Q[i] + Ql[i]);
            int j;
            for (j = 0; j < nL; j++) {
                if (de[j] == i + 1) { std::printf("%4d  %11.5f  %11.5f\n", id[pa[j] - 1], Pdp[j], Qdp[j]); break; }
                if (pa[j] == i + 1) { std::printf("%4d  %11.5f  %11.5f\n", id[de[j] - 1], Ppd[j], Qpd[j]); break; }
            }
            for (j++; j < nL; j++) {
                if (de[j] == i + 1)
                    std::printf("                                                                              %4d  %11.5f  %11.5f\n",
                                id[pa[j] - 1], Pdp[j], Qdp[j]);
                else if (pa[j] == i + 1)
                    std::printf("                                                                              %4d  %11.5f  %11.5f\n",
                                id[de[j] - 1], Ppd[j], Qpd[j]);
            }
        }
    }
    const bool to_file = o.laconic_mode || o.output_bench == GBPF_BENCH_ALL || o.output_bench == GBPF_BENCH_FILE;
    const bool to_screen = !o.laconic_mode && (o.output_bench == GBPF_BENCH_SCREEN || o.output_bench == GBPF_BENCH_ALL);
    if (to_file || to_screen) {
        double setup[5] = {0, 0, 0, 0, 0}, ph[4] = {0, 0, 0, 0};
        long long bytes[4];
        gbpf_solver_setup_times(s, setup);
        if (gbpf_solver_profile(s, 5, ph, bytes) != GBPF_OK) std::fill(ph, ph + 4, 0.0);
        tm.ybus = setup[0];
        tm.alloc = setup[1];
        tm.upload = setup[2];
        tm.stencil = setup[3];
        tm.lib = setup[4];
        tm.pq_pass = ph[0];
        tm.jac_pass = ph[1];
        tm.lin_pass = ph[2] + ph[3];
        if (to_file) write_csv(o, tm);
        if (to_screen) print_report(o, tm);
    }
    gbpf_solver_free(s);
    gbpf_grid_free(g);
    return 0;
}
