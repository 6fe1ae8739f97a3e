// gbpf_internal.h -- host-side data model shared by the libgbpf translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "gbpf.h"

namespace gbpf {

// Thread-local text of the last error (returned by gbpf_last_error).
void set_error(const std::string &msg);
const std::string &last_error();

// One grid: struct sistema / barra / ramo of the reference (GPU/sistema.h:24-126)
// as structure-of-arrays, bus indices 1-based in file order.
struct Grid {
    int nB = 0, nL = 0, nPV = 0, nPQ = 0, slack = 0;  // slack = barraVO
    double baseMVA = 100.0;
    std::vector<int> id, type;                                        // [nB]
    std::vector<double> V0, theta0, Pload, Qload, Pg, Qg, gsh, bsh;   // [nB]
    std::vector<double> Vbase;                                        // [nB]
    std::vector<int> pv, pq;                                          // 1-based, ascending
    std::vector<double> Qmin, Qmax, Vset;                             // [nPV]
    std::vector<int> de, para;                                        // [nL] 1-based
    std::vector<double> r, x, bch, tap_re, tap_im, phase;             // [nL]
    std::vector<std::string> notices;                                 // reader notices
    int ybus_form = GBPF_YBUS_CDF;                                    // branch stamps of the Ybus

    double Pliq(int k) const { return Pg[k] - Pload[k]; }
    double Qliq(int k) const { return Qg[k] - Qload[k]; }
    void rebuild_lists();  // pv / pq lists from type[]
};

// Ybus pattern (row-major CSR, sorted columns, explicit diagonal) and the
// assembly map: for each slot the contributions to sum, in the order Eigen's
// setFromTriplets sums them (branch stamps in branch order, then the shunt).
struct YPattern {
    int n = 0, nnz = 0;
    std::vector<int> rowptr, col;
    std::vector<int> diag;            // [nB] slot of (k,k)
    std::vector<int> cptr, csrc;      // per slot: stamp ids 4*branch+which, or -1-bus for the shunt
    int find(int r, int c) const;     // slot of (r,c) or -1
};
YPattern build_ypattern(const Grid &g);

// Static-pivot block LU symbolic analysis over the non-slack buses.  Block b
// (0..n-1) is bus bus_of_blk[b]; every block is a 2x2 [dP/dth dP/dV; dQ/dth dQ/dV].
// Off-diagonal factor structure is symmetric: idx(j) = up_col[up_ptr[j]..up_ptr[j+1])
// holds the blocks i > j with L(i,j) / U(j,i) != 0 (stored at the same position).
struct Symbolic {
    int n = 0;        // blocks
    int nup = 0;      // off-diagonal block positions per triangle
    std::vector<int> bus_of_blk, blk_of_bus;     // blk_of_bus[slack-1] = -1
    std::vector<int> up_ptr, up_col;
    // Crout gather lists.  Diagonal of step j: sum over dg entries of L(j,k)U(k,j);
    // dg_pos = position of j in idx(k), dg_k = k.  Off-diagonal entry p (i in idx(j)):
    // pairs (pos of j in idx(k), pos of i in idx(k)).
    std::vector<int> dg_ptr, dg_pos, dg_k;
    std::vector<long long> og_ptr;
    std::vector<int> og_a, og_b;
    std::vector<int> og_k;  // the step k of each pair (both positions lie in idx(k))
    // Level schedules: forward (factor + L solve) and backward (U solve).
    std::vector<int> flev_ptr, flev_steps, blev_ptr, blev_steps;
    // Off-diagonal entries of each forward level, flat: entries
    // fent_ptr[l]..fent_ptr[l+1] are positions fent_p[] of steps fent_j[].
    std::vector<int> fent_ptr, fent_p, fent_j;
    // Jacobian fill map over all factor block positions q in [0, n + 2*nup):
    // q < n: diagonal block q; n <= q < n+nup: L block at p = q-n (row i = up_col[p]);
    // q >= n+nup: U block at p = q-n-nup.  ysl[q] = Y slot of (row bus, col bus) or -1
    // for fill; rbus/cbus 0-based.
    std::vector<int> ysl, rbus, cbus;
    long long pairs() const { return og_ptr.empty() ? 0 : og_ptr.back(); }
};
Symbolic analyse(const Grid &g, const YPattern &y, std::string *why);

// Ordering used by analyse(): minimum degree on the bus graph, then the
// perfect elimination order of its filled graph with the shortest elimination
// tree (reduce_height: same fill, fewer levels).
std::vector<int> min_degree_order(int n, const std::vector<std::vector<int>> &adj);
std::vector<int> reduce_height(int n, const std::vector<std::vector<int>> &adj, const std::vector<int> &ord);

// Control record of one single-grid solve in device memory, written by the
// solver's graph kernels or by the one-instance batch launch below.
struct SolveCtl {
    int it;                    // Newton updates done
    int done;                  // loop finished (converged, iteration cap, failure)
    int status;                // gbpf_status
    int n_events;              // switch events recorded (may exceed the log capacity)
    unsigned long long maxG;   // bits of max|g| (non-negative doubles order as integers)
    unsigned long long maxDx;  // bits of max|dx| of the last step
    int converged;
    int pad;
};

// The single-grid solver's device arrays that a one-instance launch of the
// batch's block kernel reads (start, injections, loads) and writes (state,
// switch events, max|g| per iteration, limit-check flags, final PV limit
// flags, control record).  flat_on: device flag, nonzero when V0/th0 are the
// grid's own start (iteration 0 then comes from the topology's shared copy).
struct OneIO {
    const double *V0, *th0, *Pliq, *Qliq, *Qload;
    double *V, *th, *P, *Q;
    int *events;
    int ev_cap;
    double *hist;
    int *trig;
    int hist_cap;
    int *limQ;
    SolveCtl *ctl;
    const int *flat_on;
};
// The whole Newton solve of one grid as one persistent launch of the batch's
// block kernel (one instance, state in shared memory).  one_create fails with
// GBPF_E_UNSUPPORTED when the grid's state does not fit one block's shared
// memory; one_record enqueues the launch on `stream` (a cudaStream_t).
struct OneSolve;
gbpf_status one_create(const Grid &g, const gbpf_options &o, int device, OneSolve **out);
gbpf_status one_record(OneSolve *s, void *stream, const OneIO &io);
// The launch's LU plan (lu1: one-pass levels; narrow: one-warp levels on warp
// 0 alone; quad: FP64 one-pass levels with a block's components on four
// lanes); -1 keeps a knob.  out[0..2] = the plan in force.  Record again
// afterwards.
gbpf_status one_set_plan(OneSolve *s, int lu1, int narrow, int quad, int out[3]);
void one_free(OneSolve *s);

}  // namespace gbpf

struct gbpf_grid {
    gbpf::Grid g;
};
