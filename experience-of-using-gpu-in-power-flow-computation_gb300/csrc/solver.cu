// solver.cu -- single-grid Newton-Raphson power flow on one GPU (sm_103a).
//
// Replaces mNR (GPU/newtonRaphson.cuh:171-623) and the kernels it drives:
//   Ybus assembly         calcYbusSp_eficinte  GPU/sistema.h:705-758 (host, Eigen)
//   injections            calc{P,Q}eficiente_0based  GPU/PQcalc.cuh:177-219
//   mismatch              calcResPLim / calcResQLim  GPU/newtonRaphson.cuh:35-58
//   PV->PQ switching      chkLimQ / geraVetPV / geraVetPQ  GPU/limiteInjReat.cuh:5-75
//   Jacobian fill         SpCalcH/L/M/N  GPU/Jacobiano.cuh:252-415
//   linear solve          cusolverSpDcsrlsvqr  GPU/newtonRaphson.cuh:455-478
//   state update          attOlim / attVlim  GPU/newtonRaphson.cuh:76-119
//   convergence test      maxi + host test  GPU/newtonRaphson.cuh:390-426
// The whole loop is one CUDA graph: a prologue (reset, injections, limits,
// mismatch, test) followed by a conditional WHILE node whose body is one Newton
// iteration; the test kernel sets the loop condition on the device, so a solve
// is one graph launch and one host synchronisation.  The LU and substitutions
// run one kernel per elimination level, or for small grids every level in one
// single-block kernel (k_lu_fused).
//
// Jacobian layout: 2x2 blocks per non-slack bus ([dP/dth dP/dV; dQ/dth dQ/dV]),
// with a Q row and V column for every non-slack bus.  Buses that are PV (not at
// a Q limit) get an identity Q row and a zero V column, so PV<->PQ switches
// never change the symbolic structure; the solution of the remaining equations
// is the same as that of the reference's reduced system.
#include <cuda_runtime.h>

#include <chrono>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "blocks.cuh"
#include "gbpf_internal.h"

using gbpf::Grid;
using gbpf::set_error;
using gbpf::Symbolic;
using gbpf::YPattern;

namespace {

constexpr int kEventCap = 4096;

using Ctl = gbpf::SolveCtl;

// Every device pointer and size a kernel needs, passed by value.
struct Dev {
    int nB, nL, nnzY, slack, nPV, n, nup, max_iter, lim, hist_cap;
    double tol;
    const int *yptr, *ycol;
    double2 *yval;
    const int *cptr, *csrc;
    double2 *stamp;
    const int *br_f, *br_t;
    const double *br_r, *br_x, *br_b, *br_tre, *br_tim;
    const double *gsh, *bsh;
    double *V, *th, *cs, *sn, *P, *Q;
    double *V0, *th0, *Pliq, *Qliq;
    const double *Qload;
    const int *type;
    int *act;
    double *QliqLim;
    const int *pv_bus;
    const double *Qmin, *Qmax;
    int *limQ;
    const int *bus_of_blk, *blk_of_bus;
    const int *up_ptr, *up_col, *dg_ptr, *dg_pos, *dg_k;
    const long long *og_ptr;
    const int *og_a, *og_b;
    const int *flev_steps, *blev_steps;
    const int *fent_p, *fent_j;      // off-diagonal entries of each forward level, flat (k_factor_ent)
    const int *flev_ptr, *blev_ptr;  // level boundaries (k_lu_fused)
    int nfl, nbl;
    const int *ysl, *rbus, *cbus;
    blk4 *fac, *dinv;
    double2 *rhs, *ys, *xs;
    // FP32-LU form (precision = GBPF_PREC_FP32_IR): the factor and the
    // substitutions in FP32; fill, mismatch and update stay FP64
    float4 *fac32, *dinv32;
    float2 *ys32, *xs32;
    int fp32;
    Ctl *ctl;
    double *hist;
    int *trig;       // [hist_cap] 1 where the limit check ran (chkLimQ's "\n")
    int *events;
    // branch flows
    const int *fl_skm, *fl_smk;
    const double *fl_phi, *fl_bkm, *fl_bmk;
    double *Pdp, *Ppd, *Qdp, *Qpd;
    // metodo = denso: the dense Jacobian / LU factor [N x N], column-major, and
    // its row interchanges; dense_rule selects calcYbus's off-diagonal rule
    double *A;
    int *ipiv;
    int N, dense_rule;
    int ybus_form;  // gbpf_ybus_form of the grid
};

__device__ __forceinline__ bool stopped(const Dev &d, int guard) {
    return guard && *(volatile int *)&d.ctl->done;
}

// ------------------------------------------------------------------ Ybus
// Branch stamps of calcYbusSp_eficinte (GPU/sistema.h:708-719) and calcYbus
// (metodo = denso): (de,para) -y/conj(t), (para,de) -y/t, (de,de) y/|t|^2 + jb/2,
// (para,para) y + jb/2.  calcYbusSp_Matpower (GPU/sistema.h:760-855, .m input):
// (de,para) (-1/conj(t))/z, (para,de) (-1/t)/z, (de,de) (y + jb/2)/|t|^2.
__global__ void k_ybus_stamps(Dev d) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= d.nL) return;
    const double zr = d.br_r[b], zi = d.br_x[b];
    const double2 y = cdiv(1.0, 0.0, zr, zi);
    const double tr = d.br_tre[b], ti = d.br_tim[b];
    double a = hypot(tr, ti);
    a = 1.0 / (a * a);
    const double hb = d.br_b[b] / 2.;
    if (d.ybus_form == GBPF_YBUS_MATPOWER && !d.dense_rule) {
        const double2 uf = cdiv(-1.0, 0.0, tr, -ti), ut = cdiv(-1.0, 0.0, tr, ti);
        d.stamp[4 * b + 0] = cdiv(uf.x, uf.y, zr, zi);
        d.stamp[4 * b + 1] = cdiv(ut.x, ut.y, zr, zi);
        d.stamp[4 * b + 2] = make_double2(y.x * a, (y.y + hb) * a);
    } else {
        d.stamp[4 * b + 0] = cdiv(-y.x, -y.y, tr, -ti);
        d.stamp[4 * b + 1] = cdiv(-y.x, -y.y, tr, ti);
        d.stamp[4 * b + 2] = make_double2(a * y.x, a * y.y + hb);
    }
    d.stamp[4 * b + 3] = make_double2(y.x, y.y + hb);
}

// One slot per thread: contributions summed left to right in triplet order.
// metodo = denso builds Ybus with calcYbus (GPU/sistema.h:673-703), which
// assigns the off-diagonal entries branch by branch instead of summing them:
// there an off-diagonal slot takes its last contribution only (the two agree
// unless two branches join the same buses in opposite directions).
__global__ void k_ybus_sum(Dev d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.nnzY) return;
    double2 acc = make_double2(0, 0);
    int c0 = d.cptr[s];
    if (d.dense_rule && c0 < d.cptr[s + 1]) {
        const int src = d.csrc[c0];
        if (src >= 0 && (src & 3) < 2) c0 = d.cptr[s + 1] - 1;
    }
    for (int c = c0; c < d.cptr[s + 1]; c++) {
        const int src = d.csrc[c];
        const double2 v = src >= 0 ? d.stamp[src] : make_double2(d.gsh[-1 - src], d.bsh[-1 - src]);
        if (c == c0) acc = v;
        else { acc.x += v.x; acc.y += v.y; }
    }
    d.yval[s] = acc;
}

// ------------------------------------------------------------------ Newton kernels
// Start of a solve: flat/CDF start, limit state of initLim (GPU/limiteInjReat.cuh:188-224).
__global__ void k_reset(Dev d) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < d.nB) {
        d.V[k] = d.V0[k];
        d.th[k] = d.th0[k];
        d.QliqLim[k] = d.Qliq[k];
        d.act[k] = (d.type[k] == 0 || d.type[k] == 1);
    }
    if (k < d.nPV) d.limQ[k] = 0;
    if (k < d.hist_cap) d.trig[k] = 0;
    if (k == 0) {
        Ctl c = {};
        c.maxDx = (unsigned long long)__double_as_longlong(INFINITY);
        *d.ctl = c;
    }
}

// Unit phasors of the bus angles; also clears the mismatch maximum.
__global__ void k_phasor(Dev d, int guard) {
    if (stopped(d, guard)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) d.ctl->maxG = 0ull;
    if (k >= d.nB) return;
    double s, c;
    sincos(d.th[k], &s, &c);
    d.cs[k] = c;
    d.sn[k] = s;
}

// P, Q injections: S_k = V_k u_k conj(sum_m Y_km V_m u_m).  Four lanes per bus
// row, 16-byte loads of (G, B).
__global__ void k_pq(Dev d, int guard) {
    if (stopped(d, guard)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = t >> 2, l = t & 3;
    const bool live = k < d.nB;
    double ir = 0, ii = 0;
    if (live) {
        for (int p = d.yptr[k] + l; p < d.yptr[k + 1]; p += 4) {
            const int m = d.ycol[p];
            const double2 y = d.yval[p];
            const double em = d.V[m] * d.cs[m], fm = d.V[m] * d.sn[m];
            ir += y.x * em - y.y * fm;
            ii += y.x * fm + y.y * em;
        }
    }
    ir += __shfl_xor_sync(0xffffffffu, ir, 1);
    ii += __shfl_xor_sync(0xffffffffu, ii, 1);
    ir += __shfl_xor_sync(0xffffffffu, ir, 2);
    ii += __shfl_xor_sync(0xffffffffu, ii, 2);
    if (live && l == 0) {
        const double ek = d.V[k] * d.cs[k], fk = d.V[k] * d.sn[k];
        d.P[k] = ek * ir + fk * ii;
        d.Q[k] = fk * ir - ek * ii;
    }
}

// chkLimQ (GPU/limiteInjReat.cuh:5-40) for every PV bus, when the previous
// Newton step was small (trigger of GPU/newtonRaphson.cuh:309-314).  The
// ascending barrasPQlim merge of geraVetPQ is implicit: a bus's Q row is
// active when act[bus] = 1.
__global__ void k_limits(Dev d, int guard) {
    if (stopped(d, guard)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.nPV || !d.lim) return;
    const int it = d.ctl->it;
    if (it < 1 || it >= d.max_iter) return;
    const double mdx = __longlong_as_double((long long)d.ctl->maxDx);
    if (!(mdx < d.tol * 10.)) return;
    if (i == 0) d.trig[it] = 1;
    const int b = d.pv_bus[i];
    const double qg = d.Q[b] + d.Qload[b];
    int code = 0;
    if (qg < d.Qmin[i] - d.tol) {
        if (!d.limQ[i]) code = 1;
        else if (d.QliqLim[b] != d.Qmin[i] - d.Qload[b]) code = 2;
        d.limQ[i] = 1;
        d.QliqLim[b] = d.Qmin[i] - d.Qload[b];
    } else if (qg > d.Qmax[i] + d.tol) {
        if (!d.limQ[i]) code = 3;
        else if (d.QliqLim[b] != d.Qmax[i] - d.Qload[b]) code = 4;
        d.limQ[i] = 1;
        d.QliqLim[b] = d.Qmax[i] - d.Qload[b];
    } else {
        if (d.limQ[i]) code = 5;
        d.limQ[i] = 0;
    }
    d.act[b] = d.limQ[i];
    if (code) {
        const int e = atomicAdd(&d.ctl->n_events, 1);
        if (e < kEventCap) {
            d.events[4 * e + 0] = it;
            d.events[4 * e + 1] = b + 1;
            d.events[4 * e + 2] = i;
            d.events[4 * e + 3] = code;
        }
    }
}

// Mismatch per block: (Pliq - P, QliqLim - Q or 0 on an identity row), and max|g|.
__global__ void k_mismatch(Dev d, int guard) {
    if (stopped(d, guard)) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    double m = 0;
    if (j < d.n) {
        const int k = d.bus_of_blk[j];
        const double gp = d.Pliq[k] - d.P[k];
        const double gq = d.act[k] ? d.QliqLim[k] - d.Q[k] : 0.0;
        d.rhs[j] = make_double2(gp, gq);
        m = fmax(fabs(gp), fabs(gq));
        if (m != m) m = __longlong_as_double(0x7ff8000000000000ll);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double t = __shfl_xor_sync(0xffffffffu, m, o);
        m = (t > m || t != t) ? t : m;
    }
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&d.ctl->maxG, m);
}

// Convergence test of GPU/newtonRaphson.cuh:417-426; sets the loop condition.
__global__ void k_control(Dev d, cudaGraphConditionalHandle h, int set_cond) {
    Ctl *c = d.ctl;
    if (!c->done) {
        const double mg = __longlong_as_double((long long)c->maxG);
        if (c->it < d.hist_cap) d.hist[c->it] = mg;
        if (mg != mg) { c->status = GBPF_E_NOCONV; c->done = 1; }
        else if (mg <= d.tol) { c->converged = 1; c->done = 1; }
        else if (c->it >= d.max_iter) { c->status = GBPF_E_NOCONV; c->done = 1; }
    }
    if (set_cond) cudaGraphSetConditional(h, c->done ? 0u : 1u);
}

// Jacobian block at every factor position (fill-in positions get zeros).
// Formulas of SpCalcH/L/M/N (GPU/Jacobiano.cuh:252-344) with the angle
// difference taken from unit phasors: w = u_k conj(Y_km u_m) =
// (G cos + B sin) + j (G sin - B cos).
__global__ void k_jfill(Dev d, int guard) {
    if (stopped(d, guard)) return;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q == 0) d.ctl->maxDx = 0ull;
    if (q >= d.n + 2 * d.nup) return;
    const int s = d.ysl[q];
    blk4 blk = mk4(0, 0, 0, 0);
    if (s >= 0) {
        const int k = d.rbus[q], m = d.cbus[q];
        const double2 y = d.yval[s];
        const double Vk = d.V[k];
        const int ak = d.act[k];
        if (q < d.n) {
            const double P = d.P[k], Q = d.Q[k], v2 = Vk * Vk;
            const double H = -Q - v2 * y.y;
            if (ak) blk = mk4(H, (P + v2 * y.x) / Vk, P - v2 * y.x, (Q - v2 * y.y) / Vk);
            else blk = mk4(H, 0.0, 0.0, 1.0);
        } else {
            const int am = d.act[m];
            const double ck = d.cs[k], sk = d.sn[k], cm = d.cs[m], sm = d.sn[m];
            const double tr = y.x * cm - y.y * sm, ti = y.x * sm + y.y * cm;  // Y u_m
            const double wr = ck * tr + sk * ti, wi = sk * tr - ck * ti;      // u_k conj(Y u_m)
            const double Vm = d.V[m];
            const double H = Vk * Vm * wi, N = Vk * wr, M = -Vk * Vm * wr, L = Vk * wi;
            blk = mk4(H, am ? N : 0.0, ak ? M : 0.0, (ak && am) ? L : 0.0);
        }
    }
    if (d.fp32) d.fac32[q] = make_float4((float)blk.x, (float)blk.y, (float)blk.z, (float)blk.w);
    else d.fac[q] = blk;
}

// Factor blocks and substitution vectors in the precision of the LU.
template <typename TJ> struct SB;
template <> struct SB<double> { using b4 = blk4; using b2 = double2; };
template <> struct SB<float> { using b4 = float4; using b2 = float2; };
template <typename TJ> __device__ __forceinline__ typename SB<TJ>::b4 *fac_of(const Dev &d);
template <> __device__ __forceinline__ blk4 *fac_of<double>(const Dev &d) { return d.fac; }
template <> __device__ __forceinline__ float4 *fac_of<float>(const Dev &d) { return d.fac32; }
template <typename TJ> __device__ __forceinline__ typename SB<TJ>::b4 *dinv_of(const Dev &d);
template <> __device__ __forceinline__ blk4 *dinv_of<double>(const Dev &d) { return d.dinv; }
template <> __device__ __forceinline__ float4 *dinv_of<float>(const Dev &d) { return d.dinv32; }
template <typename TJ> __device__ __forceinline__ typename SB<TJ>::b2 *ys_of(const Dev &d);
template <> __device__ __forceinline__ double2 *ys_of<double>(const Dev &d) { return d.ys; }
template <> __device__ __forceinline__ float2 *ys_of<float>(const Dev &d) { return d.ys32; }
template <typename TJ> __device__ __forceinline__ typename SB<TJ>::b2 *xs_of(const Dev &d);
template <> __device__ __forceinline__ double2 *xs_of<double>(const Dev &d) { return d.xs; }
template <> __device__ __forceinline__ float2 *xs_of<float>(const Dev &d) { return d.xs32; }

template <typename B4> __device__ __forceinline__ B4 mmT(B4 a, B4 b) {
    B4 r;
    r.x = a.x * b.x + a.y * b.z; r.y = a.x * b.y + a.y * b.w;
    r.z = a.z * b.x + a.w * b.z; r.w = a.z * b.y + a.w * b.w;
    return r;
}
template <typename B4, typename B2> __device__ __forceinline__ B2 mvT(B4 a, B2 v) {
    B2 r;
    r.x = a.x * v.x + a.y * v.y;
    r.y = a.z * v.x + a.w * v.y;
    return r;
}
template <typename B4> __device__ __forceinline__ B4 sub4T(B4 a, B4 b) {
    a.x -= b.x; a.y -= b.y; a.z -= b.z; a.w -= b.w;
    return a;
}
template <typename B4> __device__ __forceinline__ B4 add4T(B4 a, B4 b) {
    a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w;
    return a;
}
template <typename B4> __device__ __forceinline__ B4 xsum4(B4 v, int w) {  // sum over aligned groups of w lanes
    for (int o = w >> 1; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
        v.w += __shfl_xor_sync(0xffffffffu, v.w, o);
    }
    return v;
}
template <typename B2> __device__ __forceinline__ B2 xsum2(B2 v, int w) {
    for (int o = w >> 1; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}
template <typename B4> __device__ __forceinline__ B4 bcast4(B4 v, int src) {
    v.x = __shfl_sync(0xffffffffu, v.x, src);
    v.y = __shfl_sync(0xffffffffu, v.y, src);
    v.z = __shfl_sync(0xffffffffu, v.z, src);
    v.w = __shfl_sync(0xffffffffu, v.w, src);
    return v;
}

// The pivot of step j: D_j = A_jj - sum L(j,k) U(k,j) given the gathered sum,
// its inverse and y_j = rhs_j - (gathered sum); flags a singular block.
template <typename TJ>
__device__ __forceinline__ typename SB<TJ>::b4 pivot_done(const Dev &d, int j, typename SB<TJ>::b4 acc,
                                                          typename SB<TJ>::b2 accy) {
    using B4 = typename SB<TJ>::b4;
    using B2 = typename SB<TJ>::b2;
    B4 *fac = fac_of<TJ>(d);
    const B4 D = sub4T(fac[j], acc);
    const TJ det = D.x * D.w - D.y * D.z;
    if (det == (TJ)0 || !isfinite(det)) {
        d.ctl->status = GBPF_E_SINGULAR;
        d.ctl->done = 1;
    }
    // FP64: one reciprocal, since a division is a chain of dependent FP64
    // operations, the slowest thing on a small grid's critical path.  FP32
    // keeps four divisions (cheap there; the FP32-LU form's rounding decides
    // borderline limit switches, and the golden cases were checked with it).
    B4 inv;
    if constexpr (sizeof(TJ) == 8) {
        const TJ rd = rcp_rn(det);
        inv.x = D.w * rd; inv.y = -D.y * rd; inv.z = -D.z * rd; inv.w = D.x * rd;
    } else {
        inv.x = D.w / det; inv.y = -D.y / det; inv.z = -D.z / det; inv.w = D.x / det;
    }
    fac[j] = D;
    dinv_of<TJ>(d)[j] = inv;
    const double2 r = d.rhs[j];
    B2 y;
    y.x = (TJ)r.x - accy.x;
    y.y = (TJ)r.y - accy.y;
    ys_of<TJ>(d)[j] = y;
    return inv;
}

// Crout step j on one warp (diagonal block, its inverse, the L column and U
// row of j) fused with the forward substitution y_j.
template <typename TJ>
__device__ __forceinline__ void factor_step(const Dev &d, int j, int lane) {
    using B4 = typename SB<TJ>::b4;
    using B2 = typename SB<TJ>::b2;
    B4 *fac = fac_of<TJ>(d);
    B4 *Lv = fac + d.n, *Uv = fac + d.n + d.nup;
    const B2 *ys = ys_of<TJ>(d);
    B4 acc;
    acc.x = acc.y = acc.z = acc.w = (TJ)0;
    B2 accy;
    accy.x = accy.y = (TJ)0;
    for (int t = d.dg_ptr[j] + lane; t < d.dg_ptr[j + 1]; t += 32) {
        const int a = d.dg_pos[t];
        const B4 l = Lv[a];
        acc = add4T(acc, mmT(l, Uv[a]));
        const B2 v = mvT(l, ys[d.dg_k[t]]);
        accy.x += v.x;
        accy.y += v.y;
    }
    acc = xsum4(acc, 32);
    accy = xsum2(accy, 32);
    B4 inv;
    inv.x = inv.y = inv.z = inv.w = (TJ)0;
    if (lane == 0) inv = pivot_done<TJ>(d, j, acc, accy);
    inv = bcast4(inv, 0);
    for (int p = d.up_ptr[j] + lane; p < d.up_ptr[j + 1]; p += 32) {
        B4 aL = Lv[p], aU = Uv[p];
        for (long long r = d.og_ptr[p]; r < d.og_ptr[p + 1]; r++) {
            const int a = d.og_a[r], b = d.og_b[r];
            aL = sub4T(aL, mmT(Lv[b], Uv[a]));
            aU = sub4T(aU, mmT(Lv[a], Uv[b]));
        }
        Uv[p] = aU;
        Lv[p] = mmT(aL, inv);
    }
}

// One forward level, one warp per step.
template <typename TJ>
__global__ void k_factor(Dev d, int beg, int cnt, int guard) {
    if (stopped(d, guard)) return;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= cnt) return;
    factor_step<TJ>(d, d.flev_steps[beg + w], lane);
}

// The same step for levels whose pivots carry long gather lists (the top of
// the elimination tree of large grids): one 256-thread block per step j.  The
// diagonal gather is spread over the block; each warp then takes entries of
// row j in turn and its lanes split the entry's pair list, summed with
// shuffles.
constexpr int kFacBlk = 256;
template <typename TJ>
__global__ void __launch_bounds__(kFacBlk) k_factor_blk(Dev d, int beg, int guard) {
    using B4 = typename SB<TJ>::b4;
    using B2 = typename SB<TJ>::b2;
    __shared__ B4 s_acc[kFacBlk / 32];
    __shared__ B2 s_accy[kFacBlk / 32];
    __shared__ B4 s_inv;
    __shared__ int s_stop;
    // blocks of this launch may set the stop flag (a singular pivot): read it
    // once per block so that the whole block returns or none of it does
    if (threadIdx.x == 0) s_stop = stopped(d, guard);
    __syncthreads();
    if (s_stop) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int j = d.flev_steps[beg + blockIdx.x];
    B4 *fac = fac_of<TJ>(d);
    B4 *Lv = fac + d.n, *Uv = fac + d.n + d.nup;
    const B2 *ys = ys_of<TJ>(d);
    B4 acc;
    acc.x = acc.y = acc.z = acc.w = (TJ)0;
    B2 accy;
    accy.x = accy.y = (TJ)0;
    for (int t = d.dg_ptr[j] + tid; t < d.dg_ptr[j + 1]; t += kFacBlk) {
        const int a = d.dg_pos[t];
        const B4 l = Lv[a];
        acc = add4T(acc, mmT(l, Uv[a]));
        const B2 v = mvT(l, ys[d.dg_k[t]]);
        accy.x += v.x;
        accy.y += v.y;
    }
    acc = xsum4(acc, 32);
    accy = xsum2(accy, 32);
    if (lane == 0) { s_acc[warp] = acc; s_accy[warp] = accy; }
    __syncthreads();
    if (tid == 0) {
        for (int w = 1; w < kFacBlk / 32; w++) {
            acc = add4T(acc, s_acc[w]);
            accy.x += s_accy[w].x;
            accy.y += s_accy[w].y;
        }
        s_inv = pivot_done<TJ>(d, j, acc, accy);
    }
    __syncthreads();
    const B4 inv = s_inv;
    for (int p = d.up_ptr[j] + warp; p < d.up_ptr[j + 1]; p += kFacBlk / 32) {
        B4 aL, aU;
        aL.x = aL.y = aL.z = aL.w = (TJ)0;
        aU = aL;
        for (long long r = d.og_ptr[p] + lane; r < d.og_ptr[p + 1]; r += 32) {
            const int a = d.og_a[r], b = d.og_b[r];
            aL = add4T(aL, mmT(Lv[b], Uv[a]));
            aU = add4T(aU, mmT(Lv[a], Uv[b]));
        }
        aL = xsum4(aL, 32);
        aU = xsum4(aU, 32);
        if (lane == 0) {
            Uv[p] = sub4T(Uv[p], aU);
            Lv[p] = mmT(sub4T(Lv[p], aL), inv);
        }
    }
}

// Levels with many entries per step (the top of the elimination tree of large
// grids) in two launches instead of k_factor_blk's one: k_factor_piv computes
// every pivot of the level (diagonal gather over a block, inverse, forward
// value), then k_factor_ent takes every off-diagonal entry of the level -- U(j,i)
// and the scaled L(i,j) of all its steps, flat -- one warp each across the
// whole GPU, where k_factor_blk's block walked its step's entries eight at a
// time.  Per entry the same lanes, pair order and reduction as k_factor_blk,
// so the factor is the same.
template <typename TJ>
__global__ void __launch_bounds__(kFacBlk) k_factor_piv(Dev d, int beg, int guard) {
    using B4 = typename SB<TJ>::b4;
    using B2 = typename SB<TJ>::b2;
    __shared__ B4 s_acc[kFacBlk / 32];
    __shared__ B2 s_accy[kFacBlk / 32];
    __shared__ int s_stop;
    if (threadIdx.x == 0) s_stop = stopped(d, guard);
    __syncthreads();
    if (s_stop) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int j = d.flev_steps[beg + blockIdx.x];
    B4 *fac = fac_of<TJ>(d);
    const B4 *Lv = fac + d.n, *Uv = fac + d.n + d.nup;
    const B2 *ys = ys_of<TJ>(d);
    B4 acc;
    acc.x = acc.y = acc.z = acc.w = (TJ)0;
    B2 accy;
    accy.x = accy.y = (TJ)0;
    for (int t = d.dg_ptr[j] + tid; t < d.dg_ptr[j + 1]; t += kFacBlk) {
        const int a = d.dg_pos[t];
        const B4 l = Lv[a];
        acc = add4T(acc, mmT(l, Uv[a]));
        const B2 v = mvT(l, ys[d.dg_k[t]]);
        accy.x += v.x;
        accy.y += v.y;
    }
    acc = xsum4(acc, 32);
    accy = xsum2(accy, 32);
    if (lane == 0) { s_acc[warp] = acc; s_accy[warp] = accy; }
    __syncthreads();
    if (tid == 0) {
        for (int w = 1; w < kFacBlk / 32; w++) {
            acc = add4T(acc, s_acc[w]);
            accy.x += s_accy[w].x;
            accy.y += s_accy[w].y;
        }
        (void)pivot_done<TJ>(d, j, acc, accy);
    }
}
template <typename TJ>
__global__ void k_factor_ent(Dev d, int ebeg, int ecnt, int guard) {
    using B4 = typename SB<TJ>::b4;
    if (stopped(d, guard)) return;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= ecnt) return;
    const int p = d.fent_p[ebeg + w], j = d.fent_j[ebeg + w];
    B4 *fac = fac_of<TJ>(d);
    B4 *Lv = fac + d.n, *Uv = fac + d.n + d.nup;
    B4 aL, aU;
    aL.x = aL.y = aL.z = aL.w = (TJ)0;
    aU = aL;
    for (long long r = d.og_ptr[p] + lane; r < d.og_ptr[p + 1]; r += 32) {
        const int a = d.og_a[r], b = d.og_b[r];
        aL = add4T(aL, mmT(Lv[b], Uv[a]));
        aU = add4T(aU, mmT(Lv[a], Uv[b]));
    }
    aL = xsum4(aL, 32);
    aU = xsum4(aU, 32);
    if (lane == 0) {
        Uv[p] = sub4T(Uv[p], aU);
        Lv[p] = mmT(sub4T(Lv[p], aL), dinv_of<TJ>(d)[j]);
    }
}

// Backward row j on one warp: x_j = D_j^-1 (y_j - sum_i U(j,i) x_i).
template <typename TJ>
__device__ __forceinline__ void bsolve_step(const Dev &d, int j, int lane) {
    using B4 = typename SB<TJ>::b4;
    using B2 = typename SB<TJ>::b2;
    const B4 *Uv = fac_of<TJ>(d) + d.n + d.nup;
    B2 *xs = xs_of<TJ>(d);
    B2 acc;
    acc.x = acc.y = (TJ)0;
    for (int p = d.up_ptr[j] + lane; p < d.up_ptr[j + 1]; p += 32) {
        const B2 v = mvT(Uv[p], xs[d.up_col[p]]);
        acc.x += v.x;
        acc.y += v.y;
    }
    acc = xsum2(acc, 32);
    if (lane == 0) {
        const B2 y = ys_of<TJ>(d)[j];
        B2 t;
        t.x = y.x - acc.x;
        t.y = y.y - acc.y;
        xs[j] = mvT(dinv_of<TJ>(d)[j], t);
    }
}

// One backward level, one warp per row.
template <typename TJ>
__global__ void k_bsolve(Dev d, int beg, int cnt, int guard) {
    if (stopped(d, guard)) return;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= cnt) return;
    bsolve_step<TJ>(d, d.blev_steps[beg + w], lane);
}

// Every forward level and then every backward level in one block of
// kFusedThreads, a barrier between levels, one warp per step as in
// k_factor / k_bsolve: for grids whose levels are so small that their own
// launches would cost more than their work.  A singular pivot stops it at the
// next level boundary, as the per-level launches stop (guard).
constexpr int kFusedThreads = 512;
// Largest Jacobian block order that takes k_lu_fused by default.  Measured on
// single solves (ms per solve, per-level launches -> k_lu_fused): FP32 57
// buses 0.99 -> 0.57, 118 0.79 -> 0.46, 236 5.7 -> 3.5, 472 18.5 -> 13.3, 944
// 19.8 -> 23.3, 1,888 1.35 -> 1.73; FP64 57 1.99 -> 1.76, 118 1.53 -> 1.40,
// 236 16.9 -> 19.6 (one SM's FP64 pipe is too small for more).
constexpr int kFusedMaxN32 = 600, kFusedMaxN64 = 150;
template <typename TJ>
__global__ void __launch_bounds__(kFusedThreads, 1) k_lu_fused(Dev d, int guard) {
    __shared__ int s_stop;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int W = kFusedThreads / 32;
    for (int l = 0; l < d.nfl + d.nbl; l++) {
        if (threadIdx.x == 0) s_stop = stopped(d, guard);
        __syncthreads();
        if (s_stop) return;
        if (l < d.nfl) {
            const int beg = d.flev_ptr[l], cnt = d.flev_ptr[l + 1] - beg;
            for (int w = warp; w < cnt; w += W) factor_step<TJ>(d, d.flev_steps[beg + w], lane);
        } else {
            const int lb = l - d.nfl;
            const int beg = d.blev_ptr[lb], cnt = d.blev_ptr[lb + 1] - beg;
            for (int w = warp; w < cnt; w += W) bsolve_step<TJ>(d, d.blev_steps[beg + w], lane);
        }
        __syncthreads();
    }
}

// attOlim / attVlim: theta += dx_theta, V += dx_V on active rows; max|dx|.
__global__ void k_update(Dev d, int guard) {
    if (stopped(d, guard)) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    double m = 0;
    if (j < d.n) {
        const int k = d.bus_of_blk[j];
        const double2 x = d.fp32 ? make_double2((double)d.xs32[j].x, (double)d.xs32[j].y) : d.xs[j];
        d.th[k] += x.x;
        if (d.act[k]) d.V[k] += x.y;
        m = fmax(fabs(x.x), fabs(x.y));
        if (m != m) m = __longlong_as_double(0x7ff8000000000000ll);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double t = __shfl_xor_sync(0xffffffffu, m, o);
        m = (t > m || t != t) ? t : m;
    }
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&d.ctl->maxDx, m);
    if (j == 0) d.ctl->it += 1;
}

// Branch flows of d_P_Eficiente_Sp / d_Q_Eficiente_Sp (GPU/PQcalc.cuh:523-545);
// the phase (phif) and charging (bshf) of each direction are resolved on the
// host once, so the kernel is O(nL) instead of the reference's O(nL^2) scans.
__global__ void k_flows(Dev d) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= d.nL) return;
    const int k = d.br_f[b], m = d.br_t[b];
    const double a = d.fl_phi[b] + d.th[k] - d.th[m];
    const double2 ykm = d.yval[d.fl_skm[b]], ymk = d.yval[d.fl_smk[b]];
    const double Vk = d.V[k], Vm = d.V[m];
    double sa, ca;
    sincos(a, &sa, &ca);
    d.Pdp[b] = Vk * Vk * ykm.x - Vk * Vm * ykm.x * ca - Vk * Vm * ykm.y * sa;
    d.Ppd[b] = Vm * Vm * ymk.x - Vm * Vk * ymk.x * ca - Vm * Vk * ymk.y * (-sa);
    d.Qdp[b] = -Vk * Vk * (ykm.y + d.fl_bkm[b]) + Vk * Vm * ykm.y * ca - Vk * Vm * ykm.x * sa;
    d.Qpd[b] = -Vm * Vm * (ymk.y + d.fl_bmk[b]) + Vm * Vk * ymk.y * ca - Vm * Vk * ymk.x * (-sa);
}

#include "dense.cuh"

// Largest dense system of metodo = denso: a 16384 x 16384 FP64 matrix (2 GiB),
// 8,193 buses; the right-hand side of the triangular solves sits in shared memory.
constexpr int kDenseMaxN = 16384;

// ------------------------------------------------------------------ host side
#define CK(call)                                                                     \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));          \
            return GBPF_E_CUDA;                                                      \
        }                                                                            \
    } while (0)

struct Arena {
    char *base = nullptr;
    size_t size = 0, used = 0;
    template <class T> T *take(size_t count) {
        used = (used + 255) & ~size_t(255);
        T *p = reinterpret_cast<T *>(base + used);
        used += count * sizeof(T);
        return p;
    }
};

inline int cdiv_int(long long a, int b) { return (int)((a + b - 1) / b); }

}  // namespace

struct gbpf_solver {
    Grid g;
    YPattern y;
    Symbolic S;
    gbpf_options opt{};
    int device = 0;
    cudaStream_t stream = nullptr;
    void *dmem = nullptr;
    size_t dmem_size = 0;
    Dev d{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_nodes = 0, kernels_per_iter = 0;
    Ctl last{};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // wall ms of the set-up phases: Ybus, device allocation, uploads, symbolic
    // analysis (ordering + factor structure), graph construction
    double setup_ms[5] = {0, 0, 0, 0, 0};
    // Persistent form: the whole Newton loop as one launch of the batch's
    // block kernel on this solver's arrays (gbpf::one_record), then the branch
    // flows, in a graph of its own (pexec).  form: GBPF_FORM_GRAPH or
    // GBPF_FORM_PERSISTENT, the one gbpf_solve runs.
    gbpf::OneSolve *one = nullptr;
    cudaGraph_t pgraph = nullptr;
    cudaGraphExec_t pexec = nullptr;
    int form = GBPF_FORM_GRAPH;
    int *flat_on = nullptr;   // device flag: the start is the grid's own
    int flat_on_h = 1;

    ~gbpf_solver() {
        if (pexec) cudaGraphExecDestroy(pexec);
        if (pgraph) cudaGraphDestroy(pgraph);
        if (one) gbpf::one_free(one);
        if (flat_on) cudaFree(flat_on);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (dmem) cudaFree(dmem);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }

    int nfl() const { return (int)S.flev_ptr.size() - 1; }
    int nbl() const { return (int)S.blev_ptr.size() - 1; }

    // Kernel launches of one Newton step after the mismatch: fill, factor,
    // forward and backward substitution, update.
    void launch_step(int guard) {
        const int T = 256;
        const int nq = S.n + 2 * S.nup;
        k_jfill<<<cdiv_int(nq, T), T, 0, stream>>>(d, guard);
        launch_factor_solve(guard);
        k_update<<<cdiv_int(S.n, T), T, 0, stream>>>(d, guard);
    }
    void launch_factor_solve(int guard) {
        launch_forward(guard);
        launch_backward(guard);
    }
    void launch_forward(int guard) {
        if (d.fp32) launch_forward_t<float>(guard);
        else launch_forward_t<double>(guard);
    }
    void launch_backward(int guard) {
        if (d.fp32) launch_backward_t<float>(guard);
        else launch_backward_t<double>(guard);
    }
    // Levels whose steps carry more gather work than a warp should take on
    // alone (level_heavy) run one block per step.
    // lu_fused: every level in one k_lu_fused launch (made by launch_forward;
    // launch_backward then launches nothing)
    int lu_fused = 0;
    template <typename TJ> void launch_forward_t(int guard) {
        const int T = 256, W = T / 32;
        if (lu_fused) {
            k_lu_fused<TJ><<<1, kFusedThreads, 0, stream>>>(d, guard);
            return;
        }
        for (int l = 0; l < nfl(); l++) {
            const int beg = S.flev_ptr[l], cnt = S.flev_ptr[l + 1] - beg;
            const int ebeg = S.fent_ptr[l], ecnt = S.fent_ptr[l + 1] - ebeg;
            if (level_heavy[l] && split_heavy) {
                k_factor_piv<TJ><<<cnt, kFacBlk, 0, stream>>>(d, beg, guard);
                if (ecnt) k_factor_ent<TJ><<<cdiv_int(ecnt, W), T, 0, stream>>>(d, ebeg, ecnt, guard);
            } else if (level_heavy[l]) {
                k_factor_blk<TJ><<<cnt, kFacBlk, 0, stream>>>(d, beg, guard);
            } else {
                k_factor<TJ><<<cdiv_int(cnt, W), T, 0, stream>>>(d, beg, cnt, guard);
            }
        }
    }
    template <typename TJ> void launch_backward_t(int guard) {
        const int T = 256, W = T / 32;
        if (lu_fused) return;
        for (int l = 0; l < nbl(); l++) {
            const int beg = S.blev_ptr[l], cnt = S.blev_ptr[l + 1] - beg;
            k_bsolve<TJ><<<cdiv_int(cnt, W), T, 0, stream>>>(d, beg, cnt, guard);
        }
    }
    std::vector<char> level_heavy;
    // heavy levels as two launches (k_factor_piv + k_factor_ent) rather than
    // k_factor_blk (gbpf_solver_set_lu_launch mode 3 / 1)
    int split_heavy = 1;
    // metodo = denso: dense Jacobian, blocked LU with partial pivoting, the
    // triangular solves, update
    void launch_step_dense(int guard) {
        const int T = 256;
        launch_dense_fill(guard);
        launch_dense_lu(guard);
        launch_dense_solve(guard);
        k_update<<<cdiv_int(S.n, T), T, 0, stream>>>(d, guard);
    }
    void launch_dense_fill(int guard) {
        const int T = 256, N = d.N;
        k_dzero<<<std::min(cdiv_int((long long)N * N / 2, T), 4096), T, 0, stream>>>(d, guard);
        k_dfill<<<cdiv_int(g.nB, T), T, 0, stream>>>(d, guard);
    }
    void launch_dense_lu(int guard) {
        const int T = 256, N = d.N;
        for (int k0 = 0; k0 < N; k0 += kDPanel) {
            const int k1 = std::min(N, k0 + kDPanel);
            if (N - k0 <= kDPanelSmemRows)
                k_dpanel_smem<<<1, kDPanelThreads,
                                (size_t)(N - k0 + 1) * std::min(kDPanel, N - k0) * sizeof(double), stream>>>(d, k0,
                                                                                                           guard);
            else
                k_dpanel<<<1, kDPanelThreads, 0, stream>>>(d, k0, guard);
            k_dlaswp<<<cdiv_int(N, T), T, 0, stream>>>(d, k0, guard);
            if (k1 < N) {
                k_dtrsm<<<cdiv_int(N - k1, 128), 128, 0, stream>>>(d, k0, guard);
                const int t = cdiv_int(N - k1, 64);
                k_dgemm<<<dim3(t, t), 256, 0, stream>>>(d, k0, guard);
            }
        }
    }
    void launch_dense_solve(int guard) {
        k_dsolve<<<1, kDSolveThreads, (size_t)d.N * sizeof(double), stream>>>(d, guard);
    }
    void launch_eval(int guard) {  // injections, limits, mismatch
        const int T = 256;
        k_phasor<<<cdiv_int(g.nB, T), T, 0, stream>>>(d, guard);
        k_pq<<<cdiv_int(4LL * g.nB, T), T, 0, stream>>>(d, guard);
        if (opt.lim_inj_reat && g.nPV) k_limits<<<cdiv_int(g.nPV, T), T, 0, stream>>>(d, guard);
        k_mismatch<<<cdiv_int(S.n, T), T, 0, stream>>>(d, guard);
    }

    gbpf_status build(const Grid &grid, const gbpf_options &o, int dev);
    gbpf_status build_graph();
    gbpf_status build_persistent();
    gbpf_status record_persistent();
    gbpf_status run(gbpf_result *r);
    gbpf_status finish(gbpf_result *r);
    cudaGraphExec_t active() const { return form == GBPF_FORM_PERSISTENT ? pexec : exec; }
};

gbpf_status gbpf_solver::build(const Grid &grid, const gbpf_options &o, int dev) {
    g = grid;
    opt = o;
    device = dev;
    if (g.nB < 2 || g.slack < 1) { set_error("grid needs at least two buses and one slack"); return GBPF_E_INPUT; }
    if (o.no_max_iter < 0) { set_error("no_max_iter < 0"); return GBPF_E_INPUT; }
    if (o.metodo == GBPF_METODO_DENSO && 2LL * (g.nB - 1) > kDenseMaxN) {
        set_error("metodo = denso: the dense Jacobian of " + std::to_string(g.nB) + " buses exceeds " +
                  std::to_string(kDenseMaxN) + " x " + std::to_string(kDenseMaxN) + "; use esparso");
        return GBPF_E_UNSUPPORTED;
    }
    for (int b = 0; b < g.nL; b++)
        if (g.r[b] == 0.0 && g.x[b] == 0.0) { set_error("branch with zero impedance"); return GBPF_E_INPUT; }
    using clk = std::chrono::steady_clock;
    auto ms_since = [](clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); };
    auto tp = clk::now();
    y = gbpf::build_ypattern(g);
    setup_ms[0] = ms_since(tp);
    tp = clk::now();
    std::string why;
    S = gbpf::analyse(g, y, &why);
    if (S.n != g.nB - 1) { set_error("symbolic analysis failed: " + why); return GBPF_E_INPUT; }
    setup_ms[3] = ms_since(tp);
    tp = clk::now();
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));

    const int nB = g.nB, nL = g.nL, n = S.n, nup = S.nup, nq = n + 2 * nup;
    const long long npairs = S.pairs();
    const int hist_cap = std::max(o.no_max_iter, 0) + 2;
    // flows: slot of (k,m), (m,k); phif / bshf of each branch (GPU/PQcalc.cuh:32-97)
    std::vector<int> skm(nL), smk(nL);
    std::vector<double> fphi(nL), fbkm(nL), fbmk(nL);
    for (int b = 0; b < nL; b++) {
        const int k = g.de[b], m = g.para[b];
        skm[b] = y.find(k - 1, m - 1);
        smk[b] = y.find(m - 1, k - 1);
        double ph = 0;
        bool found = false;
        for (int i = 0; i < nL; i++) if (g.de[i] == k && g.para[i] == m) { ph = g.phase[i]; found = true; break; }
        if (!found) for (int i = 0; i < nL; i++) if (g.de[i] == m && g.para[i] == k) { ph = -g.phase[i]; break; }
        fphi[b] = ph;
        auto bshf = [&](int a, int c) {
            for (int i = 0; i < nL; i++) {
                if (g.de[i] == a) { if (g.para[i] == c) return g.bch[i]; }
                else if (g.para[i] == a && g.de[i] == c) return g.bch[i];
            }
            return 0.0;
        };
        fbkm[b] = bshf(k, m);
        fbmk[b] = bshf(m, k);
    }

    // one arena for everything
    Arena A;
    for (int pass = 0; pass < 2; pass++) {
        A.used = 0;
        d = Dev{};
        d.nB = nB; d.nL = nL; d.nnzY = y.nnz; d.slack = g.slack - 1; d.nPV = g.nPV;
        d.n = n; d.nup = nup; d.max_iter = o.no_max_iter; d.lim = o.lim_inj_reat; d.tol = o.tolerancia;
        d.dense_rule = o.metodo == GBPF_METODO_DENSO;
        d.ybus_form = g.ybus_form;
        d.N = d.dense_rule ? 2 * n : 0;
        if (d.dense_rule) {
            d.A = A.take<double>((size_t)d.N * d.N);
            d.ipiv = A.take<int>(d.N);
        }
        d.hist_cap = hist_cap;
        d.yptr = A.take<int>(nB + 1); d.ycol = A.take<int>(y.nnz); d.yval = A.take<double2>(y.nnz);
        d.cptr = A.take<int>(y.nnz + 1); d.csrc = A.take<int>(y.csrc.size());
        d.stamp = A.take<double2>(4 * (size_t)nL + 1);
        d.br_f = A.take<int>(nL + 1); d.br_t = A.take<int>(nL + 1);
        d.br_r = A.take<double>(nL + 1); d.br_x = A.take<double>(nL + 1); d.br_b = A.take<double>(nL + 1);
        d.br_tre = A.take<double>(nL + 1); d.br_tim = A.take<double>(nL + 1);
        d.gsh = A.take<double>(nB); d.bsh = A.take<double>(nB);
        d.V = A.take<double>(nB); d.th = A.take<double>(nB); d.cs = A.take<double>(nB); d.sn = A.take<double>(nB);
        d.P = A.take<double>(nB); d.Q = A.take<double>(nB);
        d.V0 = A.take<double>(nB); d.th0 = A.take<double>(nB); d.Pliq = A.take<double>(nB); d.Qliq = A.take<double>(nB);
        d.Qload = A.take<double>(nB); d.type = A.take<int>(nB); d.act = A.take<int>(nB); d.QliqLim = A.take<double>(nB);
        d.pv_bus = A.take<int>(g.nPV + 1); d.Qmin = A.take<double>(g.nPV + 1); d.Qmax = A.take<double>(g.nPV + 1);
        d.limQ = A.take<int>(g.nPV + 1);
        d.bus_of_blk = A.take<int>(n); d.blk_of_bus = A.take<int>(nB);
        d.up_ptr = A.take<int>(n + 1); d.up_col = A.take<int>(nup + 1);
        d.dg_ptr = A.take<int>(n + 1); d.dg_pos = A.take<int>(nup + 1); d.dg_k = A.take<int>(nup + 1);
        d.og_ptr = A.take<long long>(nup + 1); d.og_a = A.take<int>(npairs + 1); d.og_b = A.take<int>(npairs + 1);
        d.flev_steps = A.take<int>(n); d.blev_steps = A.take<int>(n);
        d.fent_p = A.take<int>(nup + 1); d.fent_j = A.take<int>(nup + 1);
        d.flev_ptr = A.take<int>(S.flev_ptr.size()); d.blev_ptr = A.take<int>(S.blev_ptr.size());
        d.ysl = A.take<int>(nq); d.rbus = A.take<int>(nq); d.cbus = A.take<int>(nq);
        d.fp32 = o.precision == GBPF_PREC_FP32_IR && !d.dense_rule;
        if (d.fp32) {
            d.fac32 = A.take<float4>(nq); d.dinv32 = A.take<float4>(n);
            d.ys32 = A.take<float2>(n); d.xs32 = A.take<float2>(n);
        } else {
            d.fac = A.take<blk4>(nq); d.dinv = A.take<blk4>(n);
        }
        d.rhs = A.take<double2>(n); d.ys = A.take<double2>(n); d.xs = A.take<double2>(n);
        d.ctl = A.take<Ctl>(1); d.hist = A.take<double>(hist_cap); d.trig = A.take<int>(hist_cap);
        d.events = A.take<int>(4 * kEventCap);
        d.fl_skm = A.take<int>(nL + 1); d.fl_smk = A.take<int>(nL + 1);
        d.fl_phi = A.take<double>(nL + 1); d.fl_bkm = A.take<double>(nL + 1); d.fl_bmk = A.take<double>(nL + 1);
        d.Pdp = A.take<double>(nL + 1); d.Ppd = A.take<double>(nL + 1); d.Qdp = A.take<double>(nL + 1);
        d.Qpd = A.take<double>(nL + 1);
        if (pass == 0) {
            dmem_size = A.used + 256;
            cudaError_t e = cudaMalloc(&dmem, dmem_size);
            if (e != cudaSuccess) { set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e)); return GBPF_E_OOM; }
            A.base = (char *)dmem;
            A.size = dmem_size;
        }
    }
    CK(cudaMemsetAsync(dmem, 0, dmem_size, stream));
    CK(cudaStreamSynchronize(stream));
    setup_ms[1] = ms_since(tp);
    tp = clk::now();
    auto up = [&](const void *dst, const void *src, size_t bytes) -> cudaError_t {
        if (!bytes) return cudaSuccess;
        return cudaMemcpyAsync(const_cast<void *>(dst), src, bytes, cudaMemcpyHostToDevice, stream);
    };
    std::vector<int> f0(nL), t0(nL), pv0(g.nPV);
    for (int b = 0; b < nL; b++) { f0[b] = g.de[b] - 1; t0[b] = g.para[b] - 1; }
    for (int i = 0; i < g.nPV; i++) pv0[i] = g.pv[i] - 1;
    std::vector<double> pliq(nB), qliq(nB);
    for (int k = 0; k < nB; k++) { pliq[k] = g.Pliq(k); qliq[k] = g.Qliq(k); }
    CK(up(d.yptr, y.rowptr.data(), (nB + 1) * sizeof(int)));
    CK(up(d.ycol, y.col.data(), y.nnz * sizeof(int)));
    CK(up(d.cptr, y.cptr.data(), (y.nnz + 1) * sizeof(int)));
    CK(up(d.csrc, y.csrc.data(), y.csrc.size() * sizeof(int)));
    CK(up(d.br_f, f0.data(), nL * sizeof(int)));
    CK(up(d.br_t, t0.data(), nL * sizeof(int)));
    CK(up(d.br_r, g.r.data(), nL * sizeof(double)));
    CK(up(d.br_x, g.x.data(), nL * sizeof(double)));
    CK(up(d.br_b, g.bch.data(), nL * sizeof(double)));
    CK(up(d.br_tre, g.tap_re.data(), nL * sizeof(double)));
    CK(up(d.br_tim, g.tap_im.data(), nL * sizeof(double)));
    CK(up(d.gsh, g.gsh.data(), nB * sizeof(double)));
    CK(up(d.bsh, g.bsh.data(), nB * sizeof(double)));
    CK(up(d.V0, g.V0.data(), nB * sizeof(double)));
    CK(up(d.th0, g.theta0.data(), nB * sizeof(double)));
    CK(up(d.Pliq, pliq.data(), nB * sizeof(double)));
    CK(up(d.Qliq, qliq.data(), nB * sizeof(double)));
    CK(up(d.Qload, g.Qload.data(), nB * sizeof(double)));
    CK(up(d.type, g.type.data(), nB * sizeof(int)));
    CK(up(d.pv_bus, pv0.data(), g.nPV * sizeof(int)));
    CK(up(d.Qmin, g.Qmin.data(), g.nPV * sizeof(double)));
    CK(up(d.Qmax, g.Qmax.data(), g.nPV * sizeof(double)));
    CK(up(d.bus_of_blk, S.bus_of_blk.data(), n * sizeof(int)));
    CK(up(d.blk_of_bus, S.blk_of_bus.data(), nB * sizeof(int)));
    CK(up(d.up_ptr, S.up_ptr.data(), (n + 1) * sizeof(int)));
    CK(up(d.up_col, S.up_col.data(), nup * sizeof(int)));
    CK(up(d.dg_ptr, S.dg_ptr.data(), (n + 1) * sizeof(int)));
    CK(up(d.dg_pos, S.dg_pos.data(), nup * sizeof(int)));
    CK(up(d.dg_k, S.dg_k.data(), nup * sizeof(int)));
    CK(up(d.og_ptr, S.og_ptr.data(), (nup + 1) * sizeof(long long)));
    CK(up(d.og_a, S.og_a.data(), npairs * sizeof(int)));
    CK(up(d.og_b, S.og_b.data(), npairs * sizeof(int)));
    CK(up(d.flev_steps, S.flev_steps.data(), n * sizeof(int)));
    if (nup) {
        CK(up(d.fent_p, S.fent_p.data(), nup * sizeof(int)));
        CK(up(d.fent_j, S.fent_j.data(), nup * sizeof(int)));
    }
    CK(up(d.blev_steps, S.blev_steps.data(), n * sizeof(int)));
    CK(up(d.flev_ptr, S.flev_ptr.data(), S.flev_ptr.size() * sizeof(int)));
    CK(up(d.blev_ptr, S.blev_ptr.data(), S.blev_ptr.size() * sizeof(int)));
    d.nfl = nfl();
    d.nbl = nbl();
    CK(up(d.ysl, S.ysl.data(), nq * sizeof(int)));
    CK(up(d.rbus, S.rbus.data(), nq * sizeof(int)));
    CK(up(d.cbus, S.cbus.data(), nq * sizeof(int)));
    CK(up(d.fl_skm, skm.data(), nL * sizeof(int)));
    CK(up(d.fl_smk, smk.data(), nL * sizeof(int)));
    CK(up(d.fl_phi, fphi.data(), nL * sizeof(double)));
    CK(up(d.fl_bkm, fbkm.data(), nL * sizeof(double)));
    CK(up(d.fl_bmk, fbmk.data(), nL * sizeof(double)));
    CK(cudaStreamSynchronize(stream));
    setup_ms[2] = ms_since(tp);
    // forward levels whose heaviest step (diagonal gather plus the pair lists
    // of its row) exceeds heavy_work updates run one block per step (measured
    // on 236- to 15,104-bus grids: thresholds from 0 to 128 within 2 %)
    const long long heavy_work = 128;
    level_heavy.assign(nfl(), 0);
    for (int l = 0; l < nfl(); l++)
        for (int w = S.flev_ptr[l]; w < S.flev_ptr[l + 1] && !level_heavy[l]; w++) {
            const int j = S.flev_steps[w];
            long long work = S.dg_ptr[j + 1] - S.dg_ptr[j];
            for (int p = S.up_ptr[j]; p < S.up_ptr[j + 1]; p++) work += S.og_ptr[p + 1] - S.og_ptr[p];
            if (work > heavy_work) level_heavy[l] = 1;
        }
    tp = clk::now();
    // Ybus on the device, once per topology
    const int T = 256;
    if (nL) k_ybus_stamps<<<cdiv_int(nL, T), T, 0, stream>>>(d);
    k_ybus_sum<<<cdiv_int(y.nnz, T), T, 0, stream>>>(d);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    setup_ms[0] += ms_since(tp);
    tp = clk::now();
    lu_fused = !d.dense_rule && n <= (d.fp32 ? kFusedMaxN32 : kFusedMaxN64);
    gbpf_status st = build_graph();
    // the persistent form where the grid's state fits one block's shared
    // memory (metodo = esparso); it is the default in FP64.  The FP32-LU form
    // keeps the graph by default: its block kernel's one-pass FP32 levels
    // round the Newton step differently, and on a 118-bus grid with reactive
    // limits that kept every step above the limit trigger's 10 tol until
    // convergence, so no PV bus switched (the graph form's FP32 steps follow
    // the FP64 switch path there).
    if (st == GBPF_OK && !d.dense_rule) {
        const std::string keep = gbpf::last_error();
        if (build_persistent() == GBPF_OK) form = d.fp32 ? GBPF_FORM_GRAPH : GBPF_FORM_PERSISTENT;
        else set_error(keep);
    }
    setup_ms[4] = ms_since(tp);
    return st;
}

// The persistent form's graph: one launch of the batch's block kernel that
// runs the whole Newton loop on this solver's arrays, then the branch flows.
gbpf_status gbpf_solver::build_persistent() {
    gbpf_status st = gbpf::one_create(g, opt, device, &one);
    if (st != GBPF_OK) return st;
    CK(cudaMalloc(&flat_on, sizeof(int)));
    CK(cudaMemcpy(flat_on, &flat_on_h, sizeof(int), cudaMemcpyHostToDevice));
    return record_persistent();
}

// (Re)captures the persistent form's graph: the one-instance Newton launch on
// this solver's arrays, then the branch flows.
gbpf_status gbpf_solver::record_persistent() {
    if (pexec) { cudaGraphExecDestroy(pexec); pexec = nullptr; }
    if (pgraph) { cudaGraphDestroy(pgraph); pgraph = nullptr; }
    gbpf_status st = GBPF_OK;
    gbpf::OneIO io{};
    io.V0 = d.V0; io.th0 = d.th0; io.Pliq = d.Pliq; io.Qliq = d.Qliq; io.Qload = d.Qload;
    io.V = d.V; io.th = d.th; io.P = d.P; io.Q = d.Q;
    io.events = d.events;
    io.ev_cap = kEventCap;
    io.hist = d.hist;
    io.trig = d.trig;
    io.hist_cap = d.hist_cap;
    io.limQ = d.limQ;
    io.ctl = d.ctl;
    io.flat_on = flat_on;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    st = gbpf::one_record(one, stream, io);
    if (g.nL) k_flows<<<cdiv_int(g.nL, 256), 256, 0, stream>>>(d);
    cudaGraph_t gr = nullptr;
    const cudaError_t e = cudaStreamEndCapture(stream, &gr);
    if (st != GBPF_OK) { if (gr) cudaGraphDestroy(gr); return st; }
    CK(e);
    pgraph = gr;
    CK(cudaGraphInstantiate(&pexec, pgraph, 0));
    return GBPF_OK;
}

gbpf_status gbpf_solver::build_graph() {
    if (d.dense_rule) {
        CK(cudaFuncSetAttribute(k_dsolve, cudaFuncAttributeMaxDynamicSharedMemorySize, d.N * (int)sizeof(double)));
        CK(cudaFuncSetAttribute(k_dpanel_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (kDPanelSmemRows + 1) * kDPanel * (int)sizeof(double)));
    }
    CK(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle h;
    CK(cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault));
    // prologue: reset, injections, limits (inactive at iteration 0), mismatch, test
    CK(cudaStreamBeginCaptureToGraph(stream, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const int T = 256;
    k_reset<<<cdiv_int(std::max(g.nB, d.hist_cap), T), T, 0, stream>>>(d);
    launch_eval(0);
    k_control<<<1, 1, 0, stream>>>(d, h, 1);
    cudaStreamCaptureStatus cst;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    CK(cudaStreamGetCaptureInfo(stream, &cst, nullptr, nullptr, &deps, nullptr, &ndeps));
    std::vector<cudaGraphNode_t> last(deps, deps + ndeps);
    cudaGraph_t g2 = nullptr;
    CK(cudaStreamEndCapture(stream, &g2));
    // WHILE node: one Newton iteration per pass
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode;
    CK(cudaGraphAddNode(&wnode, graph, last.data(), nullptr, last.size(), &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    if (d.dense_rule) launch_step_dense(1);
    else launch_step(1);
    launch_eval(1);
    k_control<<<1, 1, 0, stream>>>(d, h, 1);
    CK(cudaStreamEndCapture(stream, &g2));
    // epilogue: branch flows of the returned state
    CK(cudaStreamBeginCaptureToGraph(stream, graph, &wnode, nullptr, 1, cudaStreamCaptureModeThreadLocal));
    if (g.nL) k_flows<<<cdiv_int(g.nL, T), T, 0, stream>>>(d);
    CK(cudaStreamEndCapture(stream, &g2));
    CK(cudaGraphInstantiate(&exec, graph, 0));
    size_t nn = 0;
    CK(cudaGraphGetNodes(graph, nullptr, &nn));
    graph_nodes = (int)nn;
    int split_levels = 0;
    if (!lu_fused && split_heavy)
        for (int l = 0; l < nfl(); l++) split_levels += level_heavy[l] && S.fent_ptr[l + 1] > S.fent_ptr[l];
    kernels_per_iter = (lu_fused ? 1 : nfl() + nbl() + split_levels) + 3 + 3 + (opt.lim_inj_reat && g.nPV ? 1 : 0) + 1;
    if (d.dense_rule) {
        const int panels = (d.N + kDPanel - 1) / kDPanel;
        kernels_per_iter = 2 + 4 * panels - 2 + 2 + 3 + (opt.lim_inj_reat && g.nPV ? 1 : 0) + 1;
    }
    return GBPF_OK;
}

gbpf_status gbpf_solver::run(gbpf_result *r) {
    CK(cudaSetDevice(device));
    CK(cudaGraphLaunch(active(), stream));
    return finish(r);
}

// Reads the control record of the solve just enqueued on the stream into
// `last` and the caller's result.
gbpf_status gbpf_solver::finish(gbpf_result *r) {
    CK(cudaMemcpyAsync(&last, d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (r) {
        r->status = last.status;
        r->converged = last.converged;
        r->iterations = last.it;
        r->n_events = last.n_events;
        std::memcpy(&r->final_mismatch, &last.maxG, sizeof(double));
        int npq = 0;
        // nPQlim = original PQ buses + PV buses at a limit (read back only when a
        // PV bus switched: every flag starts at 0)
        if (g.nPV && last.n_events > 0) {
            std::vector<int> lq(g.nPV);
            CK(cudaMemcpy(lq.data(), d.limQ, g.nPV * sizeof(int), cudaMemcpyDeviceToHost));
            for (int v : lq) npq += v;
        }
        r->nPQlim = g.nPQ + npq;
    }
    return last.status == GBPF_OK ? GBPF_OK : (gbpf_status)last.status;
}

// ---------------------------------------------------------------------- C ABI

#define ARGCHECK(c) do { if (!(c)) { set_error("invalid argument: " #c); return GBPF_E_ARG; } } while (0)

extern "C" gbpf_status gbpf_solver_create(const gbpf_grid *g, const gbpf_options *o, int device,
                                          gbpf_solver **out) {
    ARGCHECK(g && o && out);
    *out = nullptr;
    auto s = std::make_unique<gbpf_solver>();
    gbpf_status st = s->build(g->g, *o, device);
    if (st != GBPF_OK) return st;
    *out = s.release();
    return GBPF_OK;
}

extern "C" void gbpf_solver_free(gbpf_solver *s) { delete s; }

extern "C" gbpf_status gbpf_solve(gbpf_solver *s, gbpf_result *r) {
    ARGCHECK(s);
    return s->run(r);
}

extern "C" gbpf_status gbpf_solver_set_start(gbpf_solver *s, const double *V0, const double *theta0,
                                             const double *Pliq, const double *Qliq) {
    ARGCHECK(s);
    const size_t b = s->g.nB * sizeof(double);
    CK(cudaSetDevice(s->device));
    if (V0) CK(cudaMemcpyAsync(s->d.V0, V0, b, cudaMemcpyHostToDevice, s->stream));
    if (theta0) CK(cudaMemcpyAsync(s->d.th0, theta0, b, cudaMemcpyHostToDevice, s->stream));
    if ((V0 || theta0) && s->flat_on) {
        // the persistent form takes iteration 0 from the topology's shared copy
        // only while the start is the grid's own
        const bool own = (!V0 || std::equal(V0, V0 + s->g.nB, s->g.V0.begin())) &&
                         (!theta0 || std::equal(theta0, theta0 + s->g.nB, s->g.theta0.begin()));
        if ((int)own != s->flat_on_h) {
            s->flat_on_h = own;
            CK(cudaMemcpyAsync(s->flat_on, &s->flat_on_h, sizeof(int), cudaMemcpyHostToDevice, s->stream));
        }
    }
    if (Pliq) CK(cudaMemcpyAsync(s->d.Pliq, Pliq, b, cudaMemcpyHostToDevice, s->stream));
    if (Qliq) CK(cudaMemcpyAsync(s->d.Qliq, Qliq, b, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_state(gbpf_solver *s, double *V, double *theta, double *Pcalc,
                                         double *Qcalc) {
    ARGCHECK(s);
    const size_t b = s->g.nB * sizeof(double);
    CK(cudaSetDevice(s->device));
    if (V) CK(cudaMemcpyAsync(V, s->d.V, b, cudaMemcpyDeviceToHost, s->stream));
    if (theta) CK(cudaMemcpyAsync(theta, s->d.th, b, cudaMemcpyDeviceToHost, s->stream));
    if (Pcalc) CK(cudaMemcpyAsync(Pcalc, s->d.P, b, cudaMemcpyDeviceToHost, s->stream));
    if (Qcalc) CK(cudaMemcpyAsync(Qcalc, s->d.Q, b, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_events(gbpf_solver *s, int *ev, int cap, int *n) {
    ARGCHECK(s && n && (cap == 0 || ev));
    CK(cudaSetDevice(s->device));
    Ctl c;
    CK(cudaMemcpy(&c, s->d.ctl, sizeof c, cudaMemcpyDeviceToHost));
    const int have = std::min(c.n_events, kEventCap);
    std::vector<int> e(4 * (size_t)have);
    if (have) CK(cudaMemcpy(e.data(), s->d.events, e.size() * sizeof(int), cudaMemcpyDeviceToHost));
    // events of one iteration were appended in arbitrary order: sort by
    // (iteration, PV position), the order chkLimQ prints them
    std::vector<int> idx(have);
    for (int i = 0; i < have; i++) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int a, int b) {
        return e[4 * a] != e[4 * b] ? e[4 * a] < e[4 * b] : e[4 * a + 2] < e[4 * b + 2];
    });
    const int m = std::min(have, cap);
    for (int i = 0; i < m; i++) std::copy(&e[4 * idx[i]], &e[4 * idx[i]] + 4, ev + 4 * i);
    *n = m;
    return c.n_events > kEventCap ? GBPF_E_ARG : GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_history(gbpf_solver *s, double *hist, int cap, int *n) {
    ARGCHECK(s && n && (cap == 0 || hist));
    CK(cudaSetDevice(s->device));
    Ctl c;
    CK(cudaMemcpy(&c, s->d.ctl, sizeof c, cudaMemcpyDeviceToHost));
    const int have = std::min(c.it + 1, s->d.hist_cap);
    const int m = std::min(have, cap);
    if (m) CK(cudaMemcpy(hist, s->d.hist, m * sizeof(double), cudaMemcpyDeviceToHost));
    *n = m;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_triggers(gbpf_solver *s, int *trig, int cap, int *n) {
    ARGCHECK(s && n && (cap == 0 || trig));
    CK(cudaSetDevice(s->device));
    Ctl c;
    CK(cudaMemcpy(&c, s->d.ctl, sizeof c, cudaMemcpyDeviceToHost));
    const int have = std::min(c.it + 1, s->d.hist_cap);
    const int m = std::min(have, cap);
    if (m) CK(cudaMemcpy(trig, s->d.trig, m * sizeof(int), cudaMemcpyDeviceToHost));
    *n = m;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_flows(gbpf_solver *s, double *Pdp, double *Ppd, double *Qdp,
                                         double *Qpd) {
    ARGCHECK(s);
    const size_t b = s->g.nL * sizeof(double);
    CK(cudaSetDevice(s->device));
    if (Pdp) CK(cudaMemcpy(Pdp, s->d.Pdp, b, cudaMemcpyDeviceToHost));
    if (Ppd) CK(cudaMemcpy(Ppd, s->d.Ppd, b, cudaMemcpyDeviceToHost));
    if (Qdp) CK(cudaMemcpy(Qdp, s->d.Qdp, b, cudaMemcpyDeviceToHost));
    if (Qpd) CK(cudaMemcpy(Qpd, s->d.Qpd, b, cudaMemcpyDeviceToHost));
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_set_lu_launch(gbpf_solver *s, int mode) {
    ARGCHECK(s && mode >= 0 && mode <= 3);
    if (s->d.dense_rule) { set_error("metodo = denso has no level-scheduled LU"); return GBPF_E_ARG; }
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    const int fused = mode == 2 || (mode == 0 && s->S.n <= (s->d.fp32 ? kFusedMaxN32 : kFusedMaxN64));
    const int split = mode == 3 ? 0 : 1;
    if (fused == s->lu_fused && split == s->split_heavy) return GBPF_OK;
    s->lu_fused = fused;
    s->split_heavy = split;
    if (s->exec) { cudaGraphExecDestroy(s->exec); s->exec = nullptr; }
    if (s->graph) { cudaGraphDestroy(s->graph); s->graph = nullptr; }
    return s->build_graph();
}

extern "C" gbpf_status gbpf_solver_set_form(gbpf_solver *s, int form) {
    ARGCHECK(s && (form == GBPF_FORM_GRAPH || form == GBPF_FORM_PERSISTENT));
    if (form == GBPF_FORM_PERSISTENT && !s->pexec) {
        set_error("this grid has no persistent form (metodo = denso, or its state does not fit one block's shared "
                  "memory)");
        return GBPF_E_UNSUPPORTED;
    }
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    s->form = form;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_set_plan(gbpf_solver *s, int lu1, int narrow, int quad, int out[3]) {
    ARGCHECK(s);
    if (!s->one) {
        set_error("this grid has no persistent form (metodo = denso, or its state does not fit one block's shared "
                  "memory)");
        return GBPF_E_UNSUPPORTED;
    }
    CK(cudaSetDevice(s->device));
    CK(cudaStreamSynchronize(s->stream));
    gbpf_status st = gbpf::one_set_plan(s->one, lu1, narrow, quad, out);
    if (st != GBPF_OK) return st;
    return (lu1 >= 0 || narrow >= 0 || quad >= 0) ? s->record_persistent() : GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_get_form(const gbpf_solver *s, int out[3]) {
    ARGCHECK(s && out);
    out[0] = s->form;
    // persistent: the Newton kernel and the flows; graph: reset, injections
    // (+ limits), mismatch and control before the loop, flows after
    const int flows = s->g.nL ? 1 : 0;
    const int eval = 4 + (s->opt.lim_inj_reat && s->g.nPV ? 1 : 0);
    out[1] = s->form == GBPF_FORM_PERSISTENT ? 1 + flows : 1 + eval + flows;
    out[2] = s->form == GBPF_FORM_PERSISTENT ? 0 : s->kernels_per_iter;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_info(const gbpf_solver *s, long long info[8]) {
    ARGCHECK(s && info);
    info[0] = s->g.nB;
    info[1] = s->S.n;
    info[2] = s->S.nup;
    info[3] = s->S.pairs();
    info[4] = s->nfl();
    info[5] = s->nbl();
    info[6] = s->graph_nodes;
    info[7] = s->kernels_per_iter;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_time(gbpf_solver *s, int repeats, double *ms_total) {
    ARGCHECK(s && ms_total && repeats > 0);
    CK(cudaSetDevice(s->device));
    CK(cudaEventRecord(s->ev0, s->stream));
    for (int i = 0; i < repeats; i++) CK(cudaGraphLaunch(s->active(), s->stream));
    CK(cudaEventRecord(s->ev1, s->stream));
    CK(cudaEventSynchronize(s->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    *ms_total = ms;
    CK(cudaMemcpy(&s->last, s->d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    return GBPF_OK;
}

// Phase timing on the solver stream from the state the last solve left on the
// device (no host copies): 0 injections + limits + mismatch, 1 Jacobian fill,
// 2 factorisation + forward substitution (all levels), 3 backward
// substitution (all levels).  bytes[] = algorithmic bytes of one pass: every
// array a phase reads or writes counted once.
extern "C" gbpf_status gbpf_solver_setup_times(const gbpf_solver *s, double ms[5]) {
    if (!s || !ms) { set_error("invalid argument: s && ms"); return GBPF_E_ARG; }
    for (int i = 0; i < 5; i++) ms[i] = s->setup_ms[i];
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_solver_profile(gbpf_solver *s, int repeats, double ms[4], long long bytes[4]) {
    ARGCHECK(s && ms && bytes && repeats > 0);
    CK(cudaSetDevice(s->device));
    const Symbolic &S = s->S;
    const int T = 256, nq = S.n + 2 * S.nup;
    const bool dense = s->d.dense_rule;
    auto phase = [&](int ph) {
        if (ph == 0) s->launch_eval(0);
        else if (dense) {
            // metodo = denso: dense fill, the blocked LU, the triangular solves
            if (ph == 1) s->launch_dense_fill(0);
            else if (ph == 2) s->launch_dense_lu(0);
            else s->launch_dense_solve(0);
        } else if (ph == 1) k_jfill<<<cdiv_int(nq, T), T, 0, s->stream>>>(s->d, 0);
        else if (ph == 2) s->launch_forward(0);
        else s->launch_backward(0);
    };
    CK(cudaMemsetAsync(&s->d.ctl->done, 0, sizeof(int), s->stream));
    for (int ph = 0; ph < 4; ph++) {
        phase(ph);  // warm-up
        CK(cudaEventRecord(s->ev0, s->stream));
        for (int r = 0; r < repeats; r++) phase(ph);
        CK(cudaEventRecord(s->ev1, s->stream));
        CK(cudaEventSynchronize(s->ev1));
        float t = 0;
        CK(cudaEventElapsedTime(&t, s->ev0, s->ev1));
        ms[ph] = t / repeats;
    }
    CK(cudaGetLastError());
    const long long nB = s->g.nB, nnzY = s->y.nnz, n = S.n, nup = S.nup, np = S.pairs();
    // block and vector sizes of the factor's precision
    const long long b4 = s->d.fp32 ? 16 : 32, b2 = s->d.fp32 ? 8 : 16;
    // injections: Y values + columns + row pointers, V/theta/phasors, P/Q out;
    // mismatch: Pliq/Qliq/act/QliqLim, rhs out
    bytes[0] = 16 * nnzY + 4 * nnzY + 4 * (nB + 1) + 8 * nB * 2 + 16 * nB + 16 * nB + 8 * nB * 4 + 4 * nB + 16 * n;
    if (dense) {
        const long long N = s->d.N;
        // fill: the N x N matrix zeroed and written (Y values and bus state read)
        bytes[1] = 8 * N * N + 16 * nnzY + 8 * nB * 5;
        // blocked LU: each element read and written once by the panel sweep
        // (lower bound), pivots
        bytes[2] = 16 * N * N + 4 * N;
        // triangular solves: the factor read once, rhs and x
        bytes[3] = 8 * N * N + 8 * N * 2 + 4 * N;
        return GBPF_OK;
    }
    // fill: map (3 ints per block), Y values, bus state, blocks out
    bytes[1] = 12LL * nq + 16 * nnzY + 8 * nB * 5 + 4 * nB + b4 * nq;
    // factor + forward: blocks in/out, diagonal inverses, gather lists, rhs, y
    bytes[2] = 2 * b4 * nq + b4 * n + 4 * (n + 1) + 8 * nup + 4 * (nup + 1) + 8 * (nup + 1) + 8 * np + (16 + b2) * n + 4 * n;
    // backward: U blocks, inverses, columns, y in, x out
    bytes[3] = b4 * nup + b4 * n + 4 * (n + 1) + 4 * nup + 2 * b2 * n + 4 * n;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_ybus(gbpf_solver *s, int *rowptr, int *col, double *re, double *im) {
    ARGCHECK(s);
    CK(cudaSetDevice(s->device));
    const int nnz = s->y.nnz;
    std::vector<double2> v(nnz);
    CK(cudaMemcpy(v.data(), s->d.yval, nnz * sizeof(double2), cudaMemcpyDeviceToHost));
    if (rowptr) std::copy(s->y.rowptr.begin(), s->y.rowptr.end(), rowptr);
    if (col) std::copy(s->y.col.begin(), s->y.col.end(), col);
    for (int i = 0; i < nnz; i++) {
        if (re) re[i] = v[i].x;
        if (im) im[i] = v[i].y;
    }
    return GBPF_OK;
}

// Loads (V, theta) and the limit flags into the solver state, and evaluates the
// injections (no graph, plain launches on the solver stream).
static gbpf_status load_state(gbpf_solver *s, const double *V, const double *theta, const int *limQ) {
    const Grid &g = s->g;
    const size_t b = g.nB * sizeof(double);
    CK(cudaSetDevice(s->device));
    CK(cudaMemcpyAsync(s->d.V, V, b, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->d.th, theta, b, cudaMemcpyHostToDevice, s->stream));
    std::vector<int> act(g.nB);
    for (int k = 0; k < g.nB; k++) act[k] = (g.type[k] == 0 || g.type[k] == 1);
    for (int i = 0; i < g.nPV; i++) act[g.pv[i] - 1] = limQ ? (limQ[i] != 0) : 0;
    CK(cudaMemcpyAsync(s->d.act, act.data(), g.nB * sizeof(int), cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(s->d.ctl, 0, sizeof(Ctl), s->stream));
    const int T = 256;
    k_phasor<<<cdiv_int(g.nB, T), T, 0, s->stream>>>(s->d, 0);
    k_pq<<<cdiv_int(4LL * g.nB, T), T, 0, s->stream>>>(s->d, 0);
    CK(cudaGetLastError());
    // act[] must outlive the async copy
    CK(cudaStreamSynchronize(s->stream));
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_eval_pq(gbpf_solver *s, const double *V, const double *theta, double *P,
                                    double *Q) {
    ARGCHECK(s && V && theta);
    gbpf_status st = load_state(s, V, theta, nullptr);
    if (st != GBPF_OK) return st;
    const size_t b = s->g.nB * sizeof(double);
    if (P) CK(cudaMemcpy(P, s->d.P, b, cudaMemcpyDeviceToHost));
    if (Q) CK(cudaMemcpy(Q, s->d.Q, b, cudaMemcpyDeviceToHost));
    return GBPF_OK;
}

// Reference numbering of the Jacobian (Jstencil0based, GPU/esparso.h:61-178):
// P row / theta column of bus k -> k - (k > slack); Q row / V column of an
// active bus -> nB-1 + its position in the ascending list of active buses.
static void ref_numbering(const gbpf_solver *s, const int *limQ, std::vector<int> &pn, std::vector<int> &qn) {
    const Grid &g = s->g;
    const int sl = g.slack - 1;
    std::vector<int> act(g.nB);
    for (int k = 0; k < g.nB; k++) act[k] = (g.type[k] == 0 || g.type[k] == 1);
    for (int i = 0; i < g.nPV; i++) act[g.pv[i] - 1] = limQ ? (limQ[i] != 0) : 0;
    pn.assign(g.nB, -1);
    qn.assign(g.nB, -1);
    int c = 0;
    for (int k = 0; k < g.nB; k++) if (k != sl) pn[k] = k - (k > sl);
    for (int k = 0; k < g.nB; k++) if (k != sl && act[k]) qn[k] = g.nB - 1 + c++;
}

extern "C" gbpf_status gbpf_eval_jacobian(gbpf_solver *s, const double *V, const double *theta,
                                          const int *limQ, int *row, int *col, double *val, int cap,
                                          int *nnz) {
    ARGCHECK(s && V && theta && nnz);
    gbpf_status st = load_state(s, V, theta, limQ);
    if (st != GBPF_OK) return st;
    const Symbolic &S = s->S;
    const int nq = S.n + 2 * S.nup, T = 256;
    k_jfill<<<cdiv_int(nq, T), T, 0, s->stream>>>(s->d, 0);
    CK(cudaGetLastError());
    std::vector<blk4> f(nq);
    if (s->d.fp32) {
        std::vector<float4> f32(nq);
        CK(cudaMemcpyAsync(f32.data(), s->d.fac32, nq * sizeof(float4), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (int q = 0; q < nq; q++) f[q] = mk4(f32[q].x, f32[q].y, f32[q].z, f32[q].w);
    } else {
        CK(cudaMemcpyAsync(f.data(), s->d.fac, nq * sizeof(blk4), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    std::vector<int> pn, qn;
    ref_numbering(s, limQ, pn, qn);
    int m = 0;
    for (int q = 0; q < nq; q++) {
        if (S.ysl[q] < 0) continue;
        const int k = S.rbus[q], c = S.cbus[q];
        const double e[4] = {f[q].x, f[q].y, f[q].z, f[q].w};
        const int rr[4] = {pn[k], pn[k], qn[k], qn[k]}, cc[4] = {pn[c], qn[c], pn[c], qn[c]};
        for (int t = 0; t < 4; t++) {
            if (rr[t] < 0 || cc[t] < 0) continue;
            if (m < cap) { row[m] = rr[t]; col[m] = cc[t]; val[m] = e[t]; }
            m++;
        }
    }
    *nnz = m;
    return m > cap ? GBPF_E_ARG : GBPF_OK;
}

extern "C" gbpf_status gbpf_newton_step(gbpf_solver *s, const double *V, const double *theta,
                                        const int *limQ, const double *gref, double *dx) {
    ARGCHECK(s && V && theta && gref && dx);
    gbpf_status st = load_state(s, V, theta, limQ);
    if (st != GBPF_OK) return st;
    const Symbolic &S = s->S;
    std::vector<int> pn, qn;
    ref_numbering(s, limQ, pn, qn);
    std::vector<double2> rhs(S.n);
    for (int j = 0; j < S.n; j++) {
        const int k = S.bus_of_blk[j];
        rhs[j] = make_double2(gref[pn[k]], qn[k] >= 0 ? gref[qn[k]] : 0.0);
    }
    CK(cudaMemcpyAsync(s->d.rhs, rhs.data(), S.n * sizeof(double2), cudaMemcpyHostToDevice, s->stream));
    const int nq = S.n + 2 * S.nup, T = 256;
    k_jfill<<<cdiv_int(nq, T), T, 0, s->stream>>>(s->d, 0);
    s->launch_factor_solve(0);
    CK(cudaGetLastError());
    std::vector<double2> x(S.n);
    std::vector<float2> x32(s->d.fp32 ? S.n : 0);
    Ctl c;
    if (s->d.fp32) CK(cudaMemcpyAsync(x32.data(), s->d.xs32, S.n * sizeof(float2), cudaMemcpyDeviceToHost, s->stream));
    else CK(cudaMemcpyAsync(x.data(), s->d.xs, S.n * sizeof(double2), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(&c, s->d.ctl, sizeof c, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    for (size_t j = 0; j < x32.size(); j++) x[j] = make_double2(x32[j].x, x32[j].y);
    if (c.status == GBPF_E_SINGULAR) { set_error("singular Jacobian"); return GBPF_E_SINGULAR; }
    for (int j = 0; j < S.n; j++) {
        const int k = S.bus_of_blk[j];
        dx[pn[k]] = x[j].x;
        if (qn[k] >= 0) dx[qn[k]] = x[j].y;
    }
    return GBPF_OK;
}

// The graph form's Newton loop driven from the host one stage at a time: the
// same kernels (unguarded: the host decides when to stop, on the control
// record k_control writes), the device state copied back after each stage
// and handed to fn in the reference's numbering.  For verbose_mode dumps
// (GPU/newtonRaphson.cuh:284-563), so the copies and syncs do not matter.
extern "C" gbpf_status gbpf_solve_traced(gbpf_solver *s, gbpf_result *r, gbpf_trace_fn fn, void *user) {
    ARGCHECK(s && fn);
    CK(cudaSetDevice(s->device));
    const Grid &g = s->g;
    const Symbolic &S = s->S;
    const Dev &d = s->d;
    cudaStream_t st = s->stream;
    const int T = 256, nB = g.nB, nPV = g.nPV, n = S.n, nq = n + 2 * S.nup;
    const auto D2H = cudaMemcpyDeviceToHost;
    std::vector<double> P(nB), Q(nB), V(nB), th(nB), QL(nB), gv(2 * (size_t)nB), jv;
    std::vector<int> limQ(nPV + 1), pvl, pql, ev, jr, jc, pn, qn;
    std::vector<double2> x(n);
    std::vector<float2> x32(n);
    std::vector<blk4> f(nq);
    std::vector<float4> f32(nq);
    Ctl c{};
    int seen = 0, trig = 0;
    gbpf_trace t{};
    t.nB = nB;
    t.nPV = nPV;
    // state, limit flags and control record; the lists and numbering they imply
    auto read_state = [&]() -> gbpf_status {
        const size_t b = nB * sizeof(double);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(P.data(), d.P, b, D2H, st));
        CK(cudaMemcpyAsync(Q.data(), d.Q, b, D2H, st));
        CK(cudaMemcpyAsync(V.data(), d.V, b, D2H, st));
        CK(cudaMemcpyAsync(th.data(), d.th, b, D2H, st));
        CK(cudaMemcpyAsync(QL.data(), d.QliqLim, b, D2H, st));
        if (nPV) CK(cudaMemcpyAsync(limQ.data(), d.limQ, nPV * sizeof(int), D2H, st));
        CK(cudaMemcpyAsync(&c, d.ctl, sizeof(Ctl), D2H, st));
        CK(cudaStreamSynchronize(st));
        ref_numbering(s, limQ.data(), pn, qn);
        pvl.clear();
        pql.clear();
        for (int i = 0; i < nPV; i++) if (!limQ[i]) pvl.push_back(g.pv[i]);
        for (int k = 0; k < nB; k++) if (qn[k] >= 0) pql.push_back(k + 1);
        t.iteration = c.it;
        t.nPQlim = (int)pql.size();
        t.nPVlim = (int)pvl.size();
        t.n_g = nB - 1 + t.nPQlim;
        t.P = P.data(); t.Q = Q.data(); t.V = V.data(); t.theta = th.data(); t.QliqLim = QL.data();
        t.limQ = limQ.data(); t.pv_lim = pvl.data(); t.pq_lim = pql.data();
        t.g = gv.data();
        t.n_events = 0; t.events = nullptr; t.limit_check = 0;
        t.nnzJ = 0; t.jrow = t.jcol = nullptr; t.jval = nullptr;
        return GBPF_OK;
    };
    // a per-block pair vector (rhs, or the step) in the reference's numbering
    auto to_ref = [&](const double2 *v) {
        for (int j = 0; j < n; j++) {
            const int k = S.bus_of_blk[j];
            gv[pn[k]] = v[j].x;
            if (qn[k] >= 0) gv[qn[k]] = v[j].y;
        }
    };
    gbpf_status ret = GBPF_OK;
    k_reset<<<cdiv_int(std::max(nB, d.hist_cap), T), T, 0, st>>>(d);
    for (;;) {
        // injections, limit check, mismatch, convergence test
        s->launch_eval(0);
        k_control<<<1, 1, 0, st>>>(d, cudaGraphConditionalHandle{}, 0);
        if ((ret = read_state()) != GBPF_OK) return ret;
        CK(cudaMemcpy(&trig, d.trig + std::min(c.it, d.hist_cap - 1), sizeof(int), D2H));
        const int have = std::min(c.n_events, kEventCap);
        ev.assign(4 * (size_t)std::max(have - seen, 0), 0);
        if (have > seen) {
            CK(cudaMemcpy(ev.data(), d.events + 4 * (size_t)seen, ev.size() * sizeof(int), D2H));
            // appended in arbitrary order; chkLimQ prints them by PV position
            std::vector<int> idx(have - seen), e2(ev.size());
            for (size_t i = 0; i < idx.size(); i++) idx[i] = (int)i;
            std::sort(idx.begin(), idx.end(), [&](int a, int b) { return ev[4 * a + 2] < ev[4 * b + 2]; });
            for (size_t i = 0; i < idx.size(); i++) std::copy_n(&ev[4 * idx[i]], 4, &e2[4 * i]);
            ev.swap(e2);
        }
        std::vector<double2> rhs(n);
        CK(cudaMemcpy(rhs.data(), d.rhs, n * sizeof(double2), D2H));
        to_ref(rhs.data());
        t.stage = GBPF_TRACE_EVAL;
        t.done = c.done;
        t.converged = c.converged;
        std::memcpy(&t.max_g, &c.maxG, sizeof(double));
        t.limit_check = trig;
        t.n_events = (int)(ev.size() / 4);
        t.events = ev.data();
        seen = std::max(seen, have);
        fn(&t, user);
        if (c.done) break;
        // Jacobian (also in metodo = denso, whose dump is the same entries)
        k_jfill<<<cdiv_int(nq, T), T, 0, st>>>(d, 0);
        CK(cudaGetLastError());
        if (d.fp32) {
            CK(cudaMemcpyAsync(f32.data(), d.fac32, nq * sizeof(float4), D2H, st));
            CK(cudaStreamSynchronize(st));
            for (int q = 0; q < nq; q++) f[q] = mk4(f32[q].x, f32[q].y, f32[q].z, f32[q].w);
        } else {
            CK(cudaMemcpyAsync(f.data(), d.fac, nq * sizeof(blk4), D2H, st));
            CK(cudaStreamSynchronize(st));
        }
        std::vector<std::pair<long long, double>> ent;
        for (int q = 0; q < nq; q++) {
            if (S.ysl[q] < 0) continue;
            const int k = S.rbus[q], cb = S.cbus[q];
            const double e[4] = {f[q].x, f[q].y, f[q].z, f[q].w};
            const int rr[4] = {pn[k], pn[k], qn[k], qn[k]}, cc[4] = {pn[cb], qn[cb], pn[cb], qn[cb]};
            for (int u = 0; u < 4; u++)
                if (rr[u] >= 0 && cc[u] >= 0) ent.push_back({(long long)rr[u] * (nB + nB) + cc[u], e[u]});
        }
        std::sort(ent.begin(), ent.end(),
                  [](const std::pair<long long, double> &a, const std::pair<long long, double> &b) {
                      return a.first < b.first;
                  });
        jr.resize(ent.size());
        jc.resize(ent.size());
        jv.resize(ent.size());
        for (size_t i = 0; i < ent.size(); i++) {
            jr[i] = (int)(ent[i].first / (nB + nB));
            jc[i] = (int)(ent[i].first % (nB + nB));
            jv[i] = ent[i].second;
        }
        t.stage = GBPF_TRACE_JACOBIAN;
        t.nnzJ = (int)ent.size();
        t.jrow = jr.data(); t.jcol = jc.data(); t.jval = jv.data();
        t.n_events = 0; t.events = nullptr;
        fn(&t, user);
        t.nnzJ = 0; t.jrow = t.jcol = nullptr; t.jval = nullptr;
        // linear solve
        if (d.dense_rule) {
            s->launch_dense_fill(0);
            s->launch_dense_lu(0);
            s->launch_dense_solve(0);
        } else {
            s->launch_factor_solve(0);
        }
        CK(cudaGetLastError());
        if (d.fp32) {
            CK(cudaMemcpyAsync(x32.data(), d.xs32, n * sizeof(float2), D2H, st));
        } else {
            CK(cudaMemcpyAsync(x.data(), d.xs, n * sizeof(double2), D2H, st));
        }
        CK(cudaMemcpyAsync(&c, d.ctl, sizeof(Ctl), D2H, st));
        CK(cudaStreamSynchronize(st));
        if (c.done) break;  // a singular pivot ends the solve before the update, as in the graph
        if (d.fp32) for (int j = 0; j < n; j++) x[j] = make_double2(x32[j].x, x32[j].y);
        to_ref(x.data());
        t.stage = GBPF_TRACE_STEP;
        fn(&t, user);
        // update
        k_update<<<cdiv_int(n, T), T, 0, st>>>(d, 0);
        if ((ret = read_state()) != GBPF_OK) return ret;
        t.stage = GBPF_TRACE_UPDATE;
        fn(&t, user);
    }
    if (g.nL) k_flows<<<cdiv_int(g.nL, T), T, 0, st>>>(d);
    CK(cudaGetLastError());
    return s->finish(r);
}

extern "C" const char *gbpf_last_error(void) { return gbpf::last_error().c_str(); }

extern "C" const char *gbpf_status_str(gbpf_status st) {
    switch (st) {
    case GBPF_OK: return "ok";
    case GBPF_E_INPUT: return "invalid input";
    case GBPF_E_SINGULAR: return "singular Jacobian";
    case GBPF_E_NOCONV: return "no convergence";
    case GBPF_E_CUDA: return "CUDA error";
    case GBPF_E_TIMEOUT: return "device wait timed out";
    case GBPF_E_OOM: return "out of memory";
    case GBPF_E_ARG: return "invalid argument";
    case GBPF_E_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}
