// ref_harness.cpp -- runs the reference's own solve-path functions on the CPU.
//
// TEST INFRASTRUCTURE ONLY.  Linked (by oracle/ref/Makefile) against object
// files compiled unmodified from the reference's CPU/ tree:
//   reader      CPU/leitura/arquivo.cpp, CPU/leitura/cdf.cpp (byte-identical
//               logic to GPU/sistema.h:386-638)
//   Ybus        calcYbusSp_eficinte CPU/esparso/spCalcYbus.cpp:92-144
//               (same code as GPU/sistema.h:705-758); for .m input
//               calcYbusSp_Matpower CPU/esparso/spCalcYbus.cpp:4-90
//               (same code as GPU/sistema.h:760-855)
//   .m reader   CPU/leitura/m.cpp (same logic as GPU/m.h:296-622)
//   PQ          spCalcP / spCalcQ CPU/esparso/potencia/spCalcPQliq.cpp:3-45
//               (same arithmetic as GPU/PQcalc.cuh:177-219)
//   Jacobian    Jstencil0based + fillJstencil0based CPU/esparso/spCalcJac.cpp:54-224
//               (same pattern and formulas as GPU/esparso.h:61-178 and
//               GPU/Jacobiano.cuh:252-344)
//   flows       SpCalcFlux CPU/esparso/potencia/spCalcFluxPQ.cpp
// This file only replays the GPU driver's control flow
// (GPU/newtonRaphson.cuh:283-565) and its limit rules
// (GPU/limiteInjReat.cuh:5-75), which differ from the CPU tree's own driver,
// and solves each Newton step with the Eigen 3.3.7 SparseLU vendored in the
// reference (CPU/externo/Eigen) because the reference's PARDISO / cuSOLVER
// calls need MKL or a GPU.
//
// Output: one JSON object on stdout with the grid sizes, the Newton history,
// the switch events and the final state at %.17g.

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <unistd.h>

#include "estruturas.h"
#include "global.h"
#include "leitura.h"
#include "esparso/spCalcYbus.h"
#include "esparso/potencia/spCalcPQliq.h"
#include "esparso/potencia/spCalcFluxPQ.h"
#include "esparso/spCalcJac.h"
#include "externo/Eigen/Sparse"
#include "externo/Eigen/SparseLU"

void lerArquivoEAlocarMemoria(sistemaType &sistema, barraType &barra, ramoType &ramo,
                              iterativoType &iterativo);

static double maxabs(const double *v, int n) {  // maxi, GPU/newtonRaphson.cuh:24-33
    double a = 0;
    for (int i = 0; i < n; i++)
        if (std::fabs(v[i]) > a) a = std::fabs(v[i]);
    return a;
}

static void jarr(const char *name, const double *v, int n, bool last = false) {
    std::printf("\"%s\": [", name);
    for (int i = 0; i < n; i++) std::printf("%s%.17g", i ? ", " : "", v[i]);
    std::printf("]%s\n", last ? "" : ",");
}

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: ref_nr <file.cdf|.cdfx|.m> [tol] [max_iter] [lim_inj_reat] [v_inicial] [theta_inicial]\n");
        return 2;
    }
    global::arq_entrada = argv[1];
    global::tol = argc > 2 ? std::atof(argv[2]) : 1e-8;
    global::no_max_iter = argc > 3 ? std::atoi(argv[3]) : 100;
    global::lim_inj_reat = argc > 4 ? std::atoi(argv[4]) != 0 : false;
    global::v_inicial = argc > 5 ? std::atof(argv[5]) : 1.0;
    global::theta_inicial = argc > 6 ? std::atof(argv[6]) : 0.0;
    global::metodo = esparso;
    global::laconic_mode = 1;
    global::openmp = 0;

    // The reference's reader prints notices on stdout; send them to stderr so
    // that stdout carries the JSON record only.
    std::fflush(stdout);
    const int saved_stdout = dup(1);
    dup2(2, 1);

    sistemaType S{};
    barraType B{};
    ramoType R{};
    iterativoType I{};
    lerArquivoEAlocarMemoria(S, B, R, I);
    // Ybus form by input kind, as GPU/main.cu:73-82 chooses it: .m files
    // (global::isMatpower, GPU/arquivo.h:283-291) take calcYbusSp_Matpower.
    const std::string in(argv[1]);
    const size_t dot = in.find_last_of('.');
    std::string ext = dot == std::string::npos ? std::string() : in.substr(dot + 1);
    for (auto &c : ext) c = (char)std::tolower((unsigned char)c);
    if (ext == "m") calcYbusSp_Matpower(S, B, R);
    else calcYbusSp_eficinte(S, B, R);

    const int nB = S.nB, nPV = S.nPV, nPQ = S.nPQ;
    const double tol = global::tol;

    // initLim, GPU/limiteInjReat.cuh:188-224
    for (int i = 0; i < nPQ; i++) I.barrasPQlim[i] = S.barrasPQ[i];
    I.nPQlim = nPQ;
    for (int i = 0; i < nPV; i++) I.barrasPVlim[i] = S.barrasPV[i];
    I.nPVlim = nPV;
    I.ngLim = 2 * nPQ + nPV;
    for (int i = 0; i < nPV; i++) I.limQ[i] = 0;
    for (int i = 0; i < nB; i++) I.QliqLim[i] = B.Qliq[i];

    Jstencil0based(&S, &B, &R, &I);

    std::vector<double> hist;
    std::vector<int> ev;  // iteration, bus, pv position, code
    std::vector<double> dx(2 * (nPV + nPQ) + 1, 0.0);
    int it, converged = 0, singular = 0;
    double maxG = 0;
    for (it = 0; it < global::no_max_iter; it++) {
        spCalcP(S, B, R, I);
        spCalcQ(S, B, R, I);
        if (it >= 1 && global::lim_inj_reat && maxabs(dx.data(), I.ngLim) < tol * 10.) {
            // chkLimQ, GPU/limiteInjReat.cuh:5-40
            for (int i = 0; i < nPV; i++) {
                int b = S.barrasPV[i] - 1;
                double qg = I.Qcalc[b] + B.Qload[b];
                if (qg < S.limQinf[i] - tol) {
                    if (!I.limQ[i]) ev.insert(ev.end(), {it, b + 1, i, 1});
                    else if (I.QliqLim[b] != S.limQinf[i] - B.Qload[b]) ev.insert(ev.end(), {it, b + 1, i, 2});
                    I.limQ[i] = 1;
                    I.QliqLim[b] = S.limQinf[i] - B.Qload[b];
                } else if (qg > S.limQsup[i] + tol) {
                    if (!I.limQ[i]) ev.insert(ev.end(), {it, b + 1, i, 3});
                    else if (I.QliqLim[b] != S.limQsup[i] - B.Qload[b]) ev.insert(ev.end(), {it, b + 1, i, 4});
                    I.limQ[i] = 1;
                    I.QliqLim[b] = S.limQsup[i] - B.Qload[b];
                } else {
                    if (I.limQ[i]) ev.insert(ev.end(), {it, b + 1, i, 5});
                    I.limQ[i] = 0;
                }
            }
            // geraVetPV / geraVetPQ, GPU/limiteInjReat.cuh:42-75
            I.nPVlim = 0;
            for (int i = 0; i < nPV; i++)
                if (!I.limQ[i]) I.barrasPVlim[I.nPVlim++] = S.barrasPV[i];
            int a = 0, c = 0;
            for (int i = 0; i < nPV; i++) {
                if (!I.limQ[i]) continue;
                while (a < nPQ && S.barrasPQ[a] < S.barrasPV[i]) I.barrasPQlim[c++] = S.barrasPQ[a++];
                I.barrasPQlim[c++] = S.barrasPV[i];
            }
            while (a < nPQ) I.barrasPQlim[c++] = S.barrasPQ[a++];
            I.nPQlim = c;
            I.ngLim = I.nPQlim + I.nPQlim + I.nPVlim;
            // pattern rebuild, GPU/newtonRaphson.cuh:352-366
            S.spJval.clear(); S.spJsubmatType.clear(); S.cooColIndSubMatJ.clear();
            S.cooRowIndSubMatJ.clear(); S.cooColIndJ.clear(); S.cooRowIndJ.clear();
            Jstencil0based(&S, &B, &R, &I);
        }
        // calcResPLim / calcResQLim, GPU/newtonRaphson.cuh:35-58
        std::vector<double> g(I.ngLim);
        int m = 0;
        for (int k = 0; k < nB; k++)
            if (k != S.barraVO - 1) g[m++] = B.Pliq[k] - I.Pcalc[k];
        for (int i = 0; i < I.nPQlim; i++) {
            int b = I.barrasPQlim[i] - 1;
            g[m++] = I.QliqLim[b] - I.Qcalc[b];
        }
        maxG = maxabs(g.data(), I.ngLim);
        hist.push_back(maxG);
        if (maxG <= tol) { converged = 1; break; }
        fillJstencil0based(&S, &B, &R, &I);
        const int dim = I.ngLim;
        std::vector<Eigen::Triplet<double>> tr;
        tr.reserve(S.nnzJ);
        for (int p = 0; p < S.nnzJ; p++) tr.emplace_back(S.cooRowIndJ[p], S.cooColIndJ[p], S.spJval[p]);
        Eigen::SparseMatrix<double> J(dim, dim);
        J.setFromTriplets(tr.begin(), tr.end());
        Eigen::SparseLU<Eigen::SparseMatrix<double>, Eigen::COLAMDOrdering<int>> lu;
        lu.analyzePattern(J);
        lu.factorize(J);
        if (lu.info() != Eigen::Success) { singular = 1; break; }
        Eigen::Map<Eigen::VectorXd> gv(g.data(), dim);
        Eigen::VectorXd x = lu.solve(gv);
        for (int i = 0; i < dim; i++) dx[i] = x[i];
        // attOlim / attVlim, GPU/newtonRaphson.cuh:76-100
        m = 0;
        for (int k = 0; k < nB; k++)
            if (k != S.barraVO - 1) B.theta[k] += dx[m++];
        for (int i = 0; i < I.nPQlim; i++) B.V[I.barrasPQlim[i] - 1] += dx[nB - 1 + i];
    }
    if (!converged && !singular) it = global::no_max_iter;
    SpCalcFlux(&S, &B, &R);
    std::fflush(stdout);
    dup2(saved_stdout, 1);

    std::printf("{\n\"file\": \"%s\",\n", argv[1]);
    std::printf("\"nB\": %d, \"nL\": %d, \"nPV\": %d, \"nPQ\": %d, \"slack\": %d, \"nnzY\": %d,\n",
                nB, S.nL, nPV, nPQ, S.barraVO, S.nnzY);
    std::printf("\"tol\": %.17g, \"max_iter\": %d, \"lim_inj_reat\": %d,\n", tol, global::no_max_iter,
                (int)global::lim_inj_reat);
    std::printf("\"converged\": %d, \"singular\": %d, \"iterations\": %d, \"final_mismatch\": %.17g,\n",
                converged, singular, it, maxG);
    std::printf("\"nPQlim\": %d,\n", I.nPQlim);
    std::printf("\"events\": [");
    for (size_t i = 0; i < ev.size(); i += 4)
        std::printf("%s[%d, %d, %d, %d]", i ? ", " : "", ev[i], ev[i + 1], ev[i + 2], ev[i + 3]);
    std::printf("],\n");
    std::vector<double> yre(S.nnzY), yim(S.nnzY);
    for (int i = 0; i < S.nnzY; i++) { yre[i] = S.spYvalE[i].real(); yim[i] = S.spYvalE[i].imag(); }
    jarr("hist", hist.data(), (int)hist.size());
    jarr("Y_re", yre.data(), S.nnzY);
    jarr("Y_im", yim.data(), S.nnzY);
    jarr("V", B.V, nB);
    jarr("theta", B.theta, nB);
    jarr("Pcalc", I.Pcalc, nB);
    jarr("Qcalc", I.Qcalc, nB);
    jarr("Pdp", R.Pdp, S.nL);
    jarr("Ppd", R.Ppd, S.nL);
    jarr("Qdp", R.Qdp, S.nL);
    jarr("Qpd", R.Qpd, S.nL, true);
    std::printf("}\n");
    return 0;
}
