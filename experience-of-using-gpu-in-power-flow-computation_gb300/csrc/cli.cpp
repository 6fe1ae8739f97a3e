// cli.cpp -- `gbpf`, the command-line driver: the process-level drop-in for the
// reference's GPU executable (GPU/main.cu:25-216).  Reads data.txt (or the path
// given as the first argument), reads arq_entrada, solves on the GPU and prints
// what the reference prints: the option echo, the method banner, the GPU
// banner, the reactive-limit lines and max(g) trace, and the per-bus table of
// impressao2 (GPU/impressao.h:47-80).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gbpf.h"

static const char *EVENT_TEXT[6] = {
    "", "PV -> PQ (limite superior)", "PQ (limite inferior) -> PQ (limite superior)",
    "PV -> PQ (limite inferior)", "PQ (limite superior) -> PQ (limite inferior)", "PQ -> PV"};

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
    if (o.metodo != GBPF_METODO_ESPARSO && o.metodo != GBPF_METODO_NDA)
        std::fprintf(stderr, "gbpf: metodo %s runs the GPU sparse solve (no host or dense library solve)\n",
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

    gbpf_solver *s = nullptr;
    st = gbpf_solver_create(g, &o, 0, &s);
    if (st != GBPF_OK) return fail("solver setup", st);
    gbpf_result r{};
    st = gbpf_solve(s, &r);
    if (st != GBPF_OK && st != GBPF_E_NOCONV) return fail("solve", st);

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
    for (int it = 0; it <= last && it < nh; it++) {
        if (it < nt && trig[it]) {
            std::printf("\n");
            for (; e < ne && ev[4 * e] == it; e++)
                std::printf("Barra %d [%d]: %s\n", ev[4 * e + 1], ev[4 * e + 2], EVENT_TEXT[ev[4 * e + 3]]);
        }
        if (o.verbose_mode || (o.output_iter && !o.laconic_mode)) std::printf("\nmax(g) = %e", hist[it]);
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
    if (!o.laconic_mode && (o.output_bench == GBPF_BENCH_SCREEN || o.output_bench == GBPF_BENCH_ALL))
        std::printf("\n\niteracoes: %d\n", r.iterations);
    gbpf_solver_free(s);
    gbpf_grid_free(g);
    return 0;
}
