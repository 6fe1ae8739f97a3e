// batch.cu -- the whole Newton-Raphson loop of one grid instance inside one
// thread block; a persistent grid of blocks works through a queue of
// instances (load scenarios of one or several topologies) in one launch.
//
// Per instance, as in mNR (GPU/newtonRaphson.cuh:283-565): phasors, P/Q
// injections (GPU/PQcalc.cuh:177-219), the reactive-limit check
// (GPU/limiteInjReat.cuh:5-75 with the trigger of GPU/newtonRaphson.cuh:309-314),
// mismatch and convergence test (GPU/newtonRaphson.cuh:35-58,417-426), the
// Jacobian fill (GPU/Jacobiano.cuh:252-344), a static-pivot block LU with
// forward/backward substitution in place of cusolverSpDcsrlsvqr
// (GPU/newtonRaphson.cuh:455-478), and the update (GPU/newtonRaphson.cuh:76-119).
// Small topologies run one instance per warp (k_nr_warp), larger ones one per
// block (k_nr_block); the state lives in shared memory, or partly in an
// L2-resident per-block (per-warp) region where that fits more instances per
// SM (layout(), placement levels 0-3); the LU factor in shared memory when it
// fits, else in a per-block slice of a global scratch buffer.  All
// synchronisation is __syncthreads / __syncwarp between phases and LU levels:
// no kernel launches inside a solve.
//
// TJ = precision of the Jacobian, the factor and the substitutions (double:
// the oracle-matching form; float: FP32 LU with FP64 mismatch, test and update).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "blocks.cuh"
#include "gbpf_internal.h"
#include "mlp_internal.h"

using gbpf::Grid;
using gbpf::set_error;
using gbpf::Symbolic;
using gbpf::YPattern;

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
// Iteration at which an instance still running on the warp-per-instance
// kernel moves to a thread block of its own: a batch finishes when its slowest
// instance does, and a warp runs one Newton iteration several times slower
// than a block.
constexpr int kHandoffIt = 12;
// Warps (instances) per block of the warp-per-instance kernel, at most
constexpr int kWarpsMax = 16;

template <typename T> struct Blk;
template <> struct Blk<double> { using b4 = double4_32a; using b2 = double2; };
template <> struct Blk<float> { using b4 = float4; using b2 = float2; };

// Explicit fused multiply-adds, so that every use of the 2x2 block products
// below rounds the same way whatever the surrounding code lets the compiler
// contract.
__device__ __forceinline__ float fmx(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmx(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename B4> __device__ __forceinline__ B4 bm(B4 a, B4 b) {
    B4 r;
    r.x = fmx(a.x, b.x, a.y * b.z); r.y = fmx(a.x, b.y, a.y * b.w);
    r.z = fmx(a.z, b.x, a.w * b.z); r.w = fmx(a.z, b.y, a.w * b.w);
    return r;
}
template <typename B4> __device__ __forceinline__ B4 bsub(B4 a, B4 b) {
    a.x -= b.x; a.y -= b.y; a.z -= b.z; a.w -= b.w;
    return a;
}
template <typename B4> __device__ __forceinline__ B4 badd(B4 a, B4 b) {
    a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w;
    return a;
}
template <typename B4, typename B2> __device__ __forceinline__ B2 bmv(B4 a, B2 v) {
    B2 r;
    r.x = fmx(a.x, v.x, a.y * v.y);
    r.y = fmx(a.z, v.x, a.w * v.y);
    return r;
}
// v plus the v of lane (lane ^ o): one butterfly step of a sum over lanes
template <typename B2> __device__ __forceinline__ B2 b2sum_xor(B2 v, int o) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    return v;
}
template <typename B4> __device__ __forceinline__ B4 bsum_xor(B4 v, int o) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
    v.w += __shfl_xor_sync(0xffffffffu, v.w, o);
    return v;
}
template <typename B4> __device__ __forceinline__ B4 bcast(B4 v, int src) {
    v.x = __shfl_sync(0xffffffffu, v.x, src);
    v.y = __shfl_sync(0xffffffffu, v.y, src);
    v.z = __shfl_sync(0xffffffffu, v.z, src);
    v.w = __shfl_sync(0xffffffffu, v.w, src);
    return v;
}

// Topology (shared by every instance of it).  All of its read-only arrays live
// in one blob (byte offsets below) so that a block can stage the whole blob in
// shared memory with one copy when it fits.
struct TopoOff {
    int yptr, ycol, yval, type, pv_bus, Qmin, Qmax, bus_of_blk, up_ptr, up_col, dg_ptr, dg_pos, dg_k,
        og_ptr, og_a, og_b, flev_ptr, flev_steps, blev_ptr, blev_steps, ysl, rbus, cbus, fent_ptr, fent_p,
        fent_j, lvl_group, lvl_group_w, lvl_narrow, lvl_rot, og_k, yval32, lvl_group4, lvl_rot4, inj_order,
        lvl_group4w, lvl_q4w;
};
struct Topo {
    int nB, nL, n, nup, nnzY, nPV, nfl, nbl, fac_smem, blob_smem, blob_bytes;
    const char *blob;  // global copy
    const char *flat;  // the shared flat-start iteration (k_flat_start), or null
    TopoOff o;
};
// Pointers of a topology's arrays, bound to the staged (shared) or global blob.
struct TopoView {
    const int *yptr, *ycol;
    const double2 *yval;
    const int *type, *pv_bus;
    const double *Qmin, *Qmax;
    const int *bus_of_blk, *up_ptr, *up_col, *dg_ptr, *dg_pos, *dg_k, *og_ptr, *og_a, *og_b;
    const int *flev_ptr, *flev_steps, *blev_ptr, *blev_steps, *ysl, *rbus, *cbus, *fent_ptr, *fent_p, *fent_j;
    // log2 of the lanes that share one pivot / one entry / one back-substitution
    // row in the block kernel: [3 * l] pivots and [3 * l + 1] entries of
    // forward level l, [3 * l + 2] rows of backward level l
    const int *lvl_group;
    const int *lvl_group_w;  // the same for the 32 lanes of the warp kernel
    // per level: bit 0 forward level l, bit 1 backward level l has at most 32
    // pivots and 32 entries (rows): the block kernel runs it on one warp
    const int *lvl_narrow;
    // one-pass levels: lanes by which the entries of level l are rotated away
    // from its pivots (bits 0-15 the block kernel's 256 threads, bits 16-31
    // the warp's 32 lanes), so that both run side by side
    const int *lvl_rot;
    const int *og_k;  // the step k of each gather pair
    const float2 *yval32;    // Ybus values rounded to FP32 (the FP32-LU form's Jacobian)
    // lu_level1_q (FP64 one-pass levels, four lanes a block): log2 of the
    // lane quads per pivot [2 * l] and per entry [2 * l + 1] of forward level
    // l for the block kernel's 64 quads, and the threads by which the
    // entries are rotated away from the pivots (-1: a level too wide for one
    // pass of quads, which keeps one lane a block)
    const int *lvl_group4, *lvl_rot4;
    // the buses in falling order of their Ybus row's length (ties by index):
    // the order the injections take the rows in, so that the 32 rows a warp
    // walks together are about as long as each other
    const int *inj_order;
    // the same quads on 32 lanes (lu_pivots_q / lu_entries_q <32>: eight
    // quads): log2 of the quads per pivot [2 * l] and entry [2 * l + 1], and
    // 1 where forward level l fits one pass of them (else one lane a block)
    const int *lvl_group4w, *lvl_q4w;
};
__device__ __forceinline__ TopoView bind(const TopoOff &o, const char *b) {
    TopoView v;
    v.yptr = (const int *)(b + o.yptr); v.ycol = (const int *)(b + o.ycol); v.yval = (const double2 *)(b + o.yval);
    v.type = (const int *)(b + o.type); v.pv_bus = (const int *)(b + o.pv_bus);
    v.Qmin = (const double *)(b + o.Qmin); v.Qmax = (const double *)(b + o.Qmax);
    v.bus_of_blk = (const int *)(b + o.bus_of_blk); v.up_ptr = (const int *)(b + o.up_ptr);
    v.up_col = (const int *)(b + o.up_col); v.dg_ptr = (const int *)(b + o.dg_ptr);
    v.dg_pos = (const int *)(b + o.dg_pos); v.dg_k = (const int *)(b + o.dg_k);
    v.og_ptr = (const int *)(b + o.og_ptr); v.og_a = (const int *)(b + o.og_a); v.og_b = (const int *)(b + o.og_b);
    v.flev_ptr = (const int *)(b + o.flev_ptr); v.flev_steps = (const int *)(b + o.flev_steps);
    v.blev_ptr = (const int *)(b + o.blev_ptr); v.blev_steps = (const int *)(b + o.blev_steps);
    v.ysl = (const int *)(b + o.ysl); v.rbus = (const int *)(b + o.rbus); v.cbus = (const int *)(b + o.cbus);
    v.fent_ptr = (const int *)(b + o.fent_ptr); v.fent_p = (const int *)(b + o.fent_p);
    v.fent_j = (const int *)(b + o.fent_j);
    v.lvl_group = (const int *)(b + o.lvl_group);
    v.lvl_group_w = (const int *)(b + o.lvl_group_w);
    v.lvl_narrow = (const int *)(b + o.lvl_narrow);
    v.lvl_rot = (const int *)(b + o.lvl_rot);
    v.og_k = (const int *)(b + o.og_k);
    v.lvl_group4 = (const int *)(b + o.lvl_group4);
    v.lvl_rot4 = (const int *)(b + o.lvl_rot4);
    v.inj_order = (const int *)(b + o.inj_order);
    v.lvl_group4w = (const int *)(b + o.lvl_group4w);
    v.lvl_q4w = (const int *)(b + o.lvl_q4w);
    v.yval32 = (const float2 *)(b + o.yval32);
    return v;
}

struct Args {
    const Topo *topo;
    int n_inst;
    const int *inst_topo;          // [n_inst]
    const long long *inst_off;     // [n_inst] bus offset into the packed arrays
    const double *V0, *th0, *Pliq, *Qliq, *Qload;  // packed inputs
    double *V, *th, *P, *Q;                        // packed outputs
    int *iters, *status, *n_events;
    double *mism;
    int *events;                   // [n_inst * ev_cap * 4]
    int ev_cap;
    double tol;
    int max_iter, lim;
    int *counter;                  // claim counter of this launch's queue
    const int *queue;              // instance ids served by this launch
    int queue_len;
    int slice;                     // warp kernel: shared-memory bytes per warp
    char *scratch;                 // per-block factor slices when not in shared memory
    long long scratch_stride;
    int blob_region;               // bytes of dynamic shared memory reserved for a staged blob
    // Straggler hand-off.  Warp kernel: an instance still iterating when it
    // reaches iteration handoff_it (> 0) is parked -- V, theta into V/th,
    // QliqLim into Q, the PV limit flags into P, the iteration count, event
    // count and last max|dx| into iters / n_events / mism -- and its id pushed
    // to handoff_q (count in *handoff_n).  Block kernel with resume = 1: the
    // queue is handoff_q of length *handoff_n and every instance continues
    // from its parked state.  no_group = 1 makes the block kernel sum exactly
    // like the warp kernel (one lane per pivot, entry and row).
    int handoff_it;
    int *handoff_q, *handoff_n;
    int resume, no_group;
    // warp kernel: lanes grouped per pivot / entry / row on levels with few of
    // them (lvl_group_w); 0 keeps one lane per pivot, entry and row
    int warp_group;
    // block kernel: levels with at most 32 pivots and entries (rows) run on
    // warp 0 alone (lvl_narrow); 0 runs every level on the whole block
    int narrow;
    // both kernels: one pass per elimination level (lu_level1) instead of two
    int lu1;
    // block kernel, FP64 factor: levels with each 2x2 block spread over four
    // lanes (lu_level1_q, lu_pivots_q + lu_entries_q) where a level fits one
    // pass of the block's quads, instead of one lane a block
    int quad;
    // nonzero *flat_on = every instance starts from its grid's own starting
    // state, so iteration 0 takes Topo::flat (null: never)
    const int *flat_on;
    // FP32-LU form: 1 = phasors rotated by the Newton step in the update
    // (rotate_phasor), 0 = a full sincos of the new angles each iteration
    int rotate;
    // learned warm start (kind null: none).  kind[inst] = 1: the instance
    // starts from Vp/thp (the prediction) with at most warm_max_iter
    // iterations; when that run fails -- no convergence, or a PQ bus's |V|
    // ending more than warm_max_dv from the prediction (another, low-voltage
    // solution) -- it starts again from its own start in the same launch, and
    // kind becomes 2.  witers[inst] = the predicted run's iterations.  kind 0:
    // the own start (V0/th0, flat_on), max_iter iterations.
    int *kind, *witers;
    const double *Vp, *thp;
    int warm_max_iter;
    double warm_max_dv;
    // the warm start's reference iteration (FlatLayout, k_flat_start at the
    // network's mean output; null: none): iteration 0 of a predicted run
    // takes its factor -- a chord step with the Jacobian of the mean solution
    // -- in place of the instance's own Jacobian and factorisation
    const char *wref;
    // block kernel with its state in global memory (layout gs): the region of
    // block b starts at gstate + b * gstate_stride
    unsigned char *gstate;
    long long gstate_stride;
    // one-instance launches for the single-grid solver (gbpf::one_record;
    // null in batch launches): max|g| of every iteration and 1 where the
    // reactive-limit check ran (hist_cap entries), the final PV limit flags,
    // and the solve's control record
    double *hist;
    int *trig;
    int hist_cap;
    int *limq_out;
    gbpf::SolveCtl *ctl_out;
};

__host__ __device__ inline size_t align_up(size_t x, size_t a) { return (x + a - 1) & ~(a - 1); }

// Shared-memory layout of one instance (state + optionally the factor).
struct Layout {
    size_t V, th, cs, sn, ef, f32, P, Q, QL, act, lim, ys, zs, fac, total;
    size_t gtotal;  // bytes of the global state region (gs)
};
// with_zs: room for z = D^-1 y of the one-pass levels (lu_level1).  The
// inverse of diagonal block j overwrites fac[j] once the block is factored.
// gs = 1: the per-bus arrays that no thread reads for another bus's row --
// theta, P, Q, QL and, in the FP32-LU form (whose Jacobian reads the FP32
// copies), V, cos, sin -- live in a per-block region of global memory
// (offsets from its start, gtotal bytes; L2-resident) instead of shared
// memory, which halves the shared memory of an instance.  gs = 2: every
// per-bus array but the flags and y, z goes there (the phasors too, read for
// the neighbours in the injections and the Jacobian fill), leaving shared
// memory to the factor and the substitutions, the latency-critical part.
template <typename TJ>
__host__ __device__ inline Layout layout(int nB, int n, int nup, int nPV, int fac_smem, int with_zs, int gs = 0) {
    using B4 = typename Blk<TJ>::b4;
    using B2 = typename Blk<TJ>::b2;
    constexpr bool f32_form = sizeof(TJ) == 4;
    const bool vg = gs >= 2 || f32_form;  // V, cos, sin with gs
    Layout L;
    size_t o = 0, og = 0;
    auto take = [&](size_t bytes, size_t al) { o = align_up(o, al); size_t r = o; o += bytes; return r; };
    auto takeg = [&](size_t bytes, size_t al) {
        if (!gs) return take(bytes, al);
        og = align_up(og, al);
        size_t r = og;
        og += bytes;
        return r;
    };
    L.V = vg ? takeg(8 * nB, 16) : take(8 * nB, 16);
    L.th = takeg(8 * nB, 16);
    L.cs = vg ? takeg(8 * nB, 16) : take(8 * nB, 16);
    L.sn = vg ? takeg(8 * nB, 16) : take(8 * nB, 16);
    // e = V cos th, f = V sin th (FP64); cos, sin, V in FP32 for the FP32-LU form's Jacobian
    L.ef = gs >= 2 ? takeg(16 * (size_t)nB, 16) : take(16 * (size_t)nB, 16);
    L.f32 = gs >= 2 ? takeg(f32_form ? 16 * (size_t)nB : 0, 16) : take(f32_form ? 16 * (size_t)nB : 0, 16);
    L.P = takeg(8 * nB, 16); L.Q = takeg(8 * nB, 16); L.QL = takeg(8 * nB, 16);
    L.gtotal = align_up(og, 256);
    L.act = take(nB, 16); L.lim = take(4 * (size_t)(nPV + 1), 16);
    // ys: the mismatch, then (forward) the substituted right-hand side, then
    // (backward, in place) the Newton step
    L.ys = take(sizeof(B2) * n, 16);
    L.zs = with_zs ? take(sizeof(B2) * n, 16) : 0;
    const size_t nq = (size_t)n + 2 * (size_t)nup;
    L.fac = fac_smem ? take(sizeof(B4) * nq, 32) : 0;
    L.total = align_up(o, 32);
    return L;
}
// Factor slice in global scratch (used when it does not fit in shared memory).
template <typename TJ> __host__ __device__ inline size_t scratch_bytes(int n, int nup) {
    using B4 = typename Blk<TJ>::b4;
    return align_up(sizeof(B4) * ((size_t)n + 2 * (size_t)nup), 32);
}

// Iteration 0 from the grid's own starting state is the same for every
// instance of a topology: the phasors, the injections P, Q, the Jacobian and
// its factor depend on the topology and the start only; the instances differ
// in the right-hand side (their loads and generation).  k_flat_start computes
// that iteration once per topology into this layout and the warp kernel's
// instances start from it (the forward and backward substitutions with their
// own mismatch remain).
struct FlatLayout {
    size_t V0, th0, cs, sn, ef, f32, P, Q, fac, sing, total;
};
template <typename TJ> __host__ __device__ inline FlatLayout flat_layout(int nB, int nq) {
    using B4 = typename Blk<TJ>::b4;
    FlatLayout F;
    size_t o = 0;
    auto take = [&](size_t bytes, size_t al) { o = align_up(o, al); size_t r = o; o += bytes; return r; };
    F.V0 = take(8 * (size_t)nB, 16); F.th0 = take(8 * (size_t)nB, 16);
    F.cs = take(8 * (size_t)nB, 16); F.sn = take(8 * (size_t)nB, 16);
    F.ef = take(16 * (size_t)nB, 16); F.f32 = take(16 * (size_t)nB, 16);
    F.P = take(8 * (size_t)nB, 16); F.Q = take(8 * (size_t)nB, 16);
    F.fac = take(sizeof(B4) * (size_t)nq, 32);
    F.sing = take(4, 16);
    F.total = align_up(o, 256);
    return F;
}

// Maxima of |x| over FP64 values taken on their bit patterns: with the sign
// bit cleared, the unsigned order of the patterns is the order of the
// magnitudes, and every NaN pattern lies above +inf, so a NaN wins the
// maximum as the FP64 comparison chains did.  Integer instructions instead of
// FP64 compares (GB300 runs FP64 at a small fraction of its FP32 rate).
constexpr unsigned long long kAbsMask = 0x7fffffffffffffffull, kInfBits = 0x7ff0000000000000ull;
__device__ __forceinline__ unsigned long long abits(double x) {
    return (unsigned long long)__double_as_longlong(x) & kAbsMask;
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
    return a > b ? a : b;
}
__device__ __forceinline__ unsigned long long warp_umax(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) v = umax64(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ unsigned long long block_umax(unsigned long long v, unsigned long long *red) {
    v = warp_umax(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long m = red[0];
    for (int w = 1; w < kWarps; w++) m = umax64(m, red[w]);
    __syncthreads();
    return m;
}

// P + jQ of bus k: conj(sum_m Y_km e_m) times e_k, e = V (cos th + j sin th),
// with fused multiply-adds (four per Ybus entry)
__device__ __forceinline__ void injection(const int *yptr, const int *ycol, const double2 *yval, const double2 *ef,
                                          int k, double &P, double &Q) {
    double ir = 0, ii = 0;
    for (int p = yptr[k]; p < yptr[k + 1]; p++) {
        const double2 y = yval[p], u = ef[ycol[p]];
        ir = fma(y.x, u.x, ir);
        ir = fma(-y.y, u.y, ir);
        ii = fma(y.x, u.y, ii);
        ii = fma(y.y, u.x, ii);
    }
    const double ek = ef[k].x, fk = ef[k].y;
    P = fma(ek, ir, fk * ii);
    Q = fma(fk, ir, -ek * ii);
}

// FP32-LU form only: the phasor (cos, sin) of th + d from that of th.  For
// |d| <= 0.1 a rotation by d, with sin d and cos d from their Taylor series,
// cut where the next term is below 3e-19 for the step's size class; a larger
// step takes a full sincos of the new angle.  Each rotation adds a few ulps, far below the
// 1e-8 mismatch the Newton loop tests; the FP64 form keeps a full sincos.
__device__ __forceinline__ void rotate_phasor(double th_new, double d, double &c, double &s) {
    // size class from the bit pattern of |d| (integer compares)
    const unsigned long long ad = abits(d);
    const double d2 = d * d;
    double sd, cd;
    if (ad <= 0x3f1a36e2eb1c432dull) {  // |d| <= 1e-4; next terms d^5/5!, d^6/6!: below 1e-22
        sd = d * (1.0 + d2 * (-1.0 / 6.0));
        cd = 1.0 + d2 * (-0.5 + d2 * (1.0 / 24.0));
    } else if (ad <= 0x3f847ae147ae147bull) {  // |d| <= 1e-2; next terms d^9/9!, d^10/10!: below 3e-24
        sd = d * (1.0 + d2 * (-1.0 / 6.0 + d2 * (1.0 / 120.0 + d2 * (-1.0 / 5040.0))));
        cd = 1.0 + d2 * (-0.5 + d2 * (1.0 / 24.0 + d2 * (-1.0 / 720.0 + d2 * (1.0 / 40320.0))));
    } else if (ad <= 0x3fb999999999999aull) {  // |d| <= 0.1; next terms d^11/11!, d^12/12!: below 3e-19
        sd = d * (1.0 + d2 * (-1.0 / 6.0 + d2 * (1.0 / 120.0 + d2 * (-1.0 / 5040.0 + d2 * (1.0 / 362880.0)))));
        cd = 1.0 + d2 * (-0.5 + d2 * (1.0 / 24.0 + d2 * (-1.0 / 720.0 + d2 * (1.0 / 40320.0 + d2 * (-1.0 / 3628800.0)))));
    } else {
        sincos(th_new, &s, &c);
        return;
    }
    const double cn = c * cd - s * sd, sn = s * cd + c * sd;
    c = cn;
    s = sn;
}

// Diagonal Jacobian block of bus k (dP/dth, dP/dV; dQ/dth, dQ/dV at the
// injections P, Q): FP64 for the FP64 form, FP32 arithmetic for the FP32-LU
// form, whose factor holds FP32 values anyway.
template <typename TJ, typename B4>
__device__ __forceinline__ B4 diag_block(double Pk_, double Qk_, double Vk_, double2 y, int ak) {
    B4 blk;
    blk.y = blk.z = (TJ)0;
    if constexpr (sizeof(TJ) == 4) {
        const float Pk = (float)Pk_, Qk = (float)Qk_, vk = (float)Vk_, v2 = vk * vk, g = (float)y.x, b = (float)y.y;
        blk.x = -Qk - v2 * b;
        if (ak) {
            const float iv = 1.f / vk;
            blk.y = (Pk + v2 * g) * iv;
            blk.z = Pk - v2 * g;
            blk.w = (Qk - v2 * b) * iv;
        } else {
            blk.w = 1.f;
        }
    } else {
        const double v2 = Vk_ * Vk_;
        blk.x = -Qk_ - v2 * y.y;
        if (ak) {
            blk.y = (Pk_ + v2 * y.x) / Vk_;
            blk.z = Pk_ - v2 * y.x;
            blk.w = (Qk_ - v2 * y.y) / Vk_;
        } else {
            blk.w = 1.0;
        }
    }
    return blk;
}

// Diagonal block for the FP32-LU form from FP32 inputs (P, Q, V, Ybus).
template <typename B4>
__device__ __forceinline__ B4 diag_block32(float Pk, float Qk, float vk, float2 y, int ak) {
    B4 blk;
    const float v2 = vk * vk;
    blk.x = -Qk - v2 * y.y;
    blk.y = blk.z = 0.f;
    if (ak) {
        const float iv = 1.f / vk;
        blk.y = (Pk + v2 * y.x) * iv;
        blk.z = Pk - v2 * y.x;
        blk.w = (Qk - v2 * y.y) * iv;
    } else {
        blk.w = 1.f;
    }
    return blk;
}

// Phasor of bus k from th[k], V[k]: cos, sin, e = V (cos, sin) and, for the
// FP32-LU form, the FP32 copies (cos, sin, V) its Jacobian reads.  The FP64
// cos, sin are stored only where something reads them (keep_cs: the FP64
// Jacobian, the phasor rotation).
// Sine and cosine of a bus angle by the table method (P. T. P. Tang,
// "Table-lookup algorithms for elementary functions and their error
// analysis", 1991): theta = k h + d with h = 2 pi / 256 and |d| <= h / 2 (d
// from two fused multiply-adds with 2 pi split in two parts), (cos, sin)(k h)
// from a table that each batch creation copies to the device
// (trig_table_setup), (cos, sin)(d) from the Taylor polynomials to degree 6
// and 7 (the first omitted terms are below 2e-20 at |d| = pi / 256),
// combined by the angle-sum formulas: 16 FP64
// instructions and one 16-byte load, about half of what a general sincos
// spends on its range reduction, and within a few ulps of it (GB300 runs FP64
// at 1/64 of FP32, and the phasors are the largest FP64 item of an iteration).
constexpr int kTrigTab = 256;
static __device__ double2 g_trig_tab[kTrigTab];  // (cos, sin)(2 pi i / 256)
__device__ __forceinline__ void sincos_tab(double th, double *s, double *c) {
    constexpr double kInvH = 40.74366543152520595683424342336;          // 256 / (2 pi)
    constexpr double kHhi = 6.28318530717958623199592693708837 / 256.0;  // 2 pi rounded, / 256
    constexpr double kHlo = 2.44929359829470635445e-16 / 256.0;          // 2 pi - its rounding, / 256
    const double k = rint(th * kInvH);
    const double d = fma(-k, kHlo, fma(-k, kHhi, th));
    const double2 t = g_trig_tab[(int)(long long)k & (kTrigTab - 1)];
    const double d2 = d * d;
    const double cd = fma(d2, fma(d2, fma(d2, -1.0 / 720.0, 1.0 / 24.0), -0.5), 1.0);
    const double sd = fma(d * d2, fma(d2, fma(d2, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0), d);
    *c = fma(t.x, cd, -(t.y * sd));
    *s = fma(t.y, cd, t.x * sd);
}

template <typename TJ>
__device__ __forceinline__ void phasor(int k, const double *th, const double *V, double *cs, double *sn, double2 *ef,
                                       float4 *f32, bool keep_cs = true) {
    double s, c;
    sincos_tab(th[k], &s, &c);
    if (keep_cs) {
        cs[k] = c;
        sn[k] = s;
    }
    ef[k] = make_double2(V[k] * c, V[k] * s);
    if (sizeof(TJ) == 4) f32[k] = make_float4((float)c, (float)s, (float)V[k], 0.f);
}

// Jacobian block at factor position q (GPU/Jacobiano.cuh:252-344 formulas):
// diagonal blocks q < n, L / U positions after; zero at fill-in positions.
template <typename TJ>
__device__ __forceinline__ typename Blk<TJ>::b4 jac_block(const TopoView &G, int q, int n, const unsigned char *act,
                                                          const double *P, const double *Q, const double *V,
                                                          const double *cs, const double *sn, const float4 *f32) {
    using B4 = typename Blk<TJ>::b4;
    B4 blk;
    blk.x = blk.y = blk.z = blk.w = 0;
    const int sl = G.ysl[q];
    if (sl < 0) return blk;
    const int k = G.rbus[q], mb = G.cbus[q];
    const int ak = act[k];
    if constexpr (sizeof(TJ) == 4) {
        // FP32-LU form: FP32 copies of the phasors, V and Ybus
        const float4 fk = f32[k];
        const float2 y = G.yval32[sl];
        if (q < n) {
            blk = diag_block32<B4>((float)P[k], (float)Q[k], fk.z, y, ak);
        } else {
            const int am = act[mb];
            const float4 fm = f32[mb];
            const float tr = y.x * fm.x - y.y * fm.y, ti = y.x * fm.y + y.y * fm.x;
            const float wr = fk.x * tr + fk.y * ti, wi = fk.y * tr - fk.x * ti;
            blk.x = fk.z * fm.z * wi;
            if (am) blk.y = fk.z * wr;
            if (ak) blk.z = -fk.z * fm.z * wr;
            if (ak && am) blk.w = fk.z * wi;
        }
    } else {
        const double2 y = G.yval[sl];
        const double Vk = V[k];
        if (q < n) {
            blk = diag_block<TJ, B4>(P[k], Q[k], Vk, y, ak);
        } else {
            // off-diagonal entries in the precision of the factor
            const int am = act[mb];
            const TJ ck = (TJ)cs[k], sk = (TJ)sn[k], cm = (TJ)cs[mb], sm = (TJ)sn[mb];
            const TJ yr = (TJ)y.x, yi = (TJ)y.y, vk = (TJ)Vk, vm = (TJ)V[mb];
            const TJ tr = yr * cm - yi * sm, ti = yr * sm + yi * cm;
            const TJ wr = ck * tr + sk * ti, wi = sk * tr - ck * ti;
            blk.x = vk * vm * wi;
            if (am) blk.y = vk * wr;
            if (ak) blk.z = -vk * vm * wr;
            if (ak && am) blk.w = vk * wi;
        }
    }
    return blk;
}

// One elimination level, shared by both Newton kernels.  NT threads take
// part (t = 0..NT-1); a group of 2^lg of them shares one pivot (entry, row),
// strides over its gather list and sums the partial updates with shuffles
// (lane 0 of the group starts from the stored value, the others from zero, so
// lg = 0 is one thread per pivot with the list summed in order).
//
// Pivots of forward level l: diagonal block D_j (left-looking gather of
// L(j,k) U(k,j)), its inverse through one reciprocal, and y_j of the forward
// substitution.  Returns true when a pivot block is singular.
template <typename TJ, int NT>
__device__ __forceinline__ bool lu_pivots(const TopoView &G, int l, int lg, int t, typename Blk<TJ>::b4 *fac,
                                          typename Blk<TJ>::b4 *dinv, typename Blk<TJ>::b2 *ys,
                                          const typename Blk<TJ>::b4 *Lv, const typename Blk<TJ>::b4 *Uv) {
    using B4 = typename Blk<TJ>::b4;
    using B2 = typename Blk<TJ>::b2;
    const int gs = 1 << lg, gl = t & (gs - 1), ng = NT >> lg;
    const int beg = G.flev_ptr[l], cnt = G.flev_ptr[l + 1] - beg;
    bool sing = false;
    for (int b0 = 0; b0 < cnt; b0 += ng) {
        const int w = b0 + (t >> lg);
        const bool on = w < cnt;
        const int j = on ? G.flev_steps[beg + w] : 0;
        B4 D;
        B2 yj;
        D.x = D.y = D.z = D.w = (TJ)0;
        yj.x = yj.y = (TJ)0;
        if (on && gl == 0) {
            D = fac[j];
            yj = ys[j];
        }
        if (on)
            for (int q = G.dg_ptr[j] + gl; q < G.dg_ptr[j + 1]; q += gs) {
                const int p = G.dg_pos[q];
                const B4 lj = Lv[p];
                D = bsub(D, bm(lj, Uv[p]));
                const B2 v = bmv(lj, ys[G.dg_k[q]]);
                yj.x -= v.x;
                yj.y -= v.y;
            }
        for (int o = gs >> 1; o > 0; o >>= 1) {
            D = bsum_xor(D, o);
            yj = b2sum_xor(yj, o);
        }
        if (on && gl == 0) {
            const TJ det = D.x * D.w - D.y * D.z;
            sing |= (det == (TJ)0 || !isfinite(det));
            const TJ rd = rcp_rn(det);
            B4 inv;
            inv.x = D.w * rd; inv.y = -D.y * rd; inv.z = -D.z * rd; inv.w = D.x * rd;
            dinv[j] = inv;  // the slot of D_j when dinv aliases the factor's diagonal
            ys[j] = yj;
        }
    }
    return sing;
}

// Off-diagonal entries of forward level l: U(j,i) and L(i,j) = (...) D_j^-1.
template <typename TJ, int NT>
__device__ __forceinline__ void lu_entries(const TopoView &G, int l, int lg, int t, const typename Blk<TJ>::b4 *dinv,
                                           typename Blk<TJ>::b4 *Lv, typename Blk<TJ>::b4 *Uv) {
    using B4 = typename Blk<TJ>::b4;
    const int gs = 1 << lg, gl = t & (gs - 1), ng = NT >> lg;
    const int beg = G.fent_ptr[l], cnt = G.fent_ptr[l + 1] - beg;
    for (int b0 = 0; b0 < cnt; b0 += ng) {
        const int e = b0 + (t >> lg);
        const bool on = e < cnt;
        const int p = on ? G.fent_p[beg + e] : 0, j = on ? G.fent_j[beg + e] : 0;
        B4 aL, aU;
        aL.x = aL.y = aL.z = aL.w = (TJ)0;
        aU = aL;
        if (on && gl == 0) { aL = Lv[p]; aU = Uv[p]; }
        if (on)
            for (int r = G.og_ptr[p] + gl; r < G.og_ptr[p + 1]; r += gs) {
                const int x = G.og_a[r], y = G.og_b[r];
                aL = bsub(aL, bm(Lv[y], Uv[x]));
                aU = bsub(aU, bm(Lv[x], Uv[y]));
            }
        for (int o = gs >> 1; o > 0; o >>= 1) {
            aL = bsum_xor(aL, o);
            aU = bsum_xor(aU, o);
        }
        if (on && gl == 0) {
            Uv[p] = aU;
            Lv[p] = bm(aL, dinv[j]);
        }
    }
}

// Rows of backward level l: x_j = D_j^-1 (y_j - sum_i U(j,i) x_i), in place in ys.
template <typename TJ, int NT>
__device__ __forceinline__ void back_rows(const TopoView &G, int l, int lg, int t, const typename Blk<TJ>::b4 *dinv,
                                          const typename Blk<TJ>::b4 *Uv, typename Blk<TJ>::b2 *ys) {
    using B2 = typename Blk<TJ>::b2;
    const int gs = 1 << lg, gl = t & (gs - 1), ng = NT >> lg;
    const int beg = G.blev_ptr[l], cnt = G.blev_ptr[l + 1] - beg;
    for (int b0 = 0; b0 < cnt; b0 += ng) {
        const int w = b0 + (t >> lg);
        const bool on = w < cnt;
        const int j = on ? G.blev_steps[beg + w] : 0;
        B2 acc;
        acc.x = acc.y = (TJ)0;
        if (on && gl == 0) acc = ys[j];
        if (on)
            for (int p = G.up_ptr[j] + gl; p < G.up_ptr[j + 1]; p += gs) {
                const B2 v = bmv(Uv[p], ys[G.up_col[p]]);
                acc.x -= v.x;
                acc.y -= v.y;
            }
        for (int o = gs >> 1; o > 0; o >>= 1) acc = b2sum_xor(acc, o);
        if (on && gl == 0) ys[j] = bmv(dinv[j], acc);
    }
}

// Forward substitution alone on forward level l with a factor made earlier
// (two-pass form, L scaled): y_j -= sum_k L(j,k) y_k, summed exactly as the
// y part of lu_pivots with the same lane groups, so the result is the one the
// fused factor-and-substitute pass gives.
template <typename TJ, int NT>
__device__ __forceinline__ void fwd_rows(const TopoView &G, int l, int lg, int t, const typename Blk<TJ>::b4 *Lv,
                                         typename Blk<TJ>::b2 *ys) {
    using B2 = typename Blk<TJ>::b2;
    const int gs = 1 << lg, gl = t & (gs - 1), ng = NT >> lg;
    const int beg = G.flev_ptr[l], cnt = G.flev_ptr[l + 1] - beg;
    for (int b0 = 0; b0 < cnt; b0 += ng) {
        const int w = b0 + (t >> lg);
        const bool on = w < cnt;
        const int j = on ? G.flev_steps[beg + w] : 0;
        B2 yj;
        yj.x = yj.y = (TJ)0;
        if (on && gl == 0) yj = ys[j];
        if (on)
            for (int q = G.dg_ptr[j] + gl; q < G.dg_ptr[j + 1]; q += gs) {
                const B2 v = bmv(Lv[G.dg_pos[q]], ys[G.dg_k[q]]);
                yj.x -= v.x;
                yj.y -= v.y;
            }
        for (int o = gs >> 1; o > 0; o >>= 1) yj = b2sum_xor(yj, o);
        if (on && gl == 0) ys[j] = yj;
    }
}

// One-pass level l: pivots and off-diagonal entries of the level together.
// L is kept unscaled, Lt(i,k) = L(i,k) D_k, so no entry of a level waits for
// the inverse of its own pivot; consumers apply D_k^-1 themselves:
//   D_j    = A_jj   - sum_k Lt(j,k) D_k^-1 U(k,j)
//   y_j    = b_j    - sum_k Lt(j,k) z_k,   z_k = D_k^-1 y_k
//   Lt(i,j) = A_ij  - sum_k Lt(i,k) D_k^-1 U(k,j)
//   U(j,i)  = A_ji  - sum_k Lt(j,k) D_k^-1 U(k,i)
// (every k of a gather lies on an earlier level).  The backward
// substitution is unchanged.  Entries run on lanes rotated by `rot` (a
// multiple of their group size) so that they overlap the pivots' lanes as
// little as possible.  Returns true when a pivot block is singular.
template <typename TJ, int NT>
__device__ __forceinline__ bool lu_level1(const TopoView &G, int l, int lgp, int lge, int rot, int t,
                                          typename Blk<TJ>::b4 *fac, typename Blk<TJ>::b4 *dinv,
                                          typename Blk<TJ>::b2 *ys, typename Blk<TJ>::b2 *zs,
                                          typename Blk<TJ>::b4 *Lv, typename Blk<TJ>::b4 *Uv) {
    using B4 = typename Blk<TJ>::b4;
    using B2 = typename Blk<TJ>::b2;
    bool sing = false;
    {
        const int gs = 1 << lgp, gl = t & (gs - 1), ng = NT >> lgp;
        const int beg = G.flev_ptr[l], cnt = G.flev_ptr[l + 1] - beg;
        for (int b0 = 0; b0 < cnt; b0 += ng) {
            const int w = b0 + (t >> lgp);
            const bool on = w < cnt;
            const int j = on ? G.flev_steps[beg + w] : 0;
            B4 D;
            B2 yj;
            D.x = D.y = D.z = D.w = (TJ)0;
            yj.x = yj.y = (TJ)0;
            if (on && gl == 0) {
                D = fac[j];
                yj = ys[j];
            }
            if (on)
                for (int q = G.dg_ptr[j] + gl; q < G.dg_ptr[j + 1]; q += gs) {
                    const int p = G.dg_pos[q], k = G.dg_k[q];
                    const B4 lt = Lv[p];
                    D = bsub(D, bm(lt, bm(dinv[k], Uv[p])));
                    const B2 v = bmv(lt, zs[k]);
                    yj.x -= v.x;
                    yj.y -= v.y;
                }
            for (int o = gs >> 1; o > 0; o >>= 1) {
                D = bsum_xor(D, o);
                yj = b2sum_xor(yj, o);
            }
            if (on && gl == 0) {
                const TJ det = D.x * D.w - D.y * D.z;
                sing |= (det == (TJ)0 || !isfinite(det));
                const TJ rd = rcp_rn(det);
                B4 inv;
                inv.x = D.w * rd; inv.y = -D.y * rd; inv.z = -D.z * rd; inv.w = D.x * rd;
                dinv[j] = inv;
                ys[j] = yj;
                zs[j] = bmv(inv, yj);
            }
        }
    }
    {
        const int te = (t + rot) & (NT - 1);
        const int gs = 1 << lge, gl = te & (gs - 1), ng = NT >> lge;
        const int beg = G.fent_ptr[l], cnt = G.fent_ptr[l + 1] - beg;
        for (int b0 = 0; b0 < cnt; b0 += ng) {
            const int e = b0 + (te >> lge);
            const bool on = e < cnt;
            const int p = on ? G.fent_p[beg + e] : 0;
            B4 aL, aU;
            aL.x = aL.y = aL.z = aL.w = (TJ)0;
            aU = aL;
            if (on && gl == 0) { aL = Lv[p]; aU = Uv[p]; }
            if (on)
                for (int r = G.og_ptr[p] + gl; r < G.og_ptr[p + 1]; r += gs) {
                    const int x = G.og_a[r], y = G.og_b[r];
                    const B4 dk = dinv[G.og_k[r]];
                    aL = bsub(aL, bm(Lv[y], bm(dk, Uv[x])));
                    aU = bsub(aU, bm(Lv[x], bm(dk, Uv[y])));
                }
            for (int o = gs >> 1; o > 0; o >>= 1) {
                aL = bsum_xor(aL, o);
                aU = bsum_xor(aU, o);
            }
            if (on && gl == 0) {
                Uv[p] = aU;
                Lv[p] = aL;
            }
        }
    }
    return sing;
}

// FP64 one-pass level l (the equations of lu_level1) with each 2x2 block
// spread over a quad of four lanes: lane c = 2 r + s of the quad holds
// component (r, s) of every block it touches.  GB300's FP64 pipe takes a
// warp instruction 16 cycles whatever lanes are active, so the product of two
// blocks costs each lane one multiply and one fused multiply-add (rounded as
// bm(): fma(A[r][0], B[0][s], A[r][1] B[1][s])) instead of four of each on
// one lane, and a group sum one add a step instead of four.  The gathers,
// lists and order of accumulation are lu_level1's, over logical lanes of four
// threads (NT / 4 of them, 2^lg to a pivot or entry).  Returns true when a
// pivot block is singular.
template <int NT>
__device__ __forceinline__ bool lu_level1_q(const TopoView &G, int l, int lgp, int lge, int rot, int t,
                                            double4_32a *fac, double4_32a *dinv, double2 *ys, double2 *zs,
                                            double4_32a *Lv, double4_32a *Uv) {
    const int c = t & 3, r = c >> 1, s = c & 1, qb = (t & 31) & ~3;
    const unsigned qm = 0xfu << qb;  // the quad's lanes, which always run together
    const int sA0 = qb + 2 * r, sA1 = sA0 + 1, sB0 = qb + s, sB1 = qb + 2 + s;
    auto comp = [&](const double4_32a *p) { return ((const double *)p)[c]; };
    // component c of A B, A and B held a component a lane; a0, a1 = row r of A
    auto qmul = [&](double a, double b, double &a0, double &a1) {
        a0 = __shfl_sync(qm, a, sA0);
        a1 = __shfl_sync(qm, a, sA1);
        const double b0 = __shfl_sync(qm, b, sB0), b1 = __shfl_sync(qm, b, sB1);
        return __fma_rn(a0, b0, a1 * b1);
    };
    bool sing = false;
    {
        const int tl = t >> 2, gs = 1 << lgp, gl = tl & (gs - 1), ng = (NT >> 2) >> lgp;
        const int beg = G.flev_ptr[l], cnt = G.flev_ptr[l + 1] - beg;
        for (int b0 = 0; b0 < cnt; b0 += ng) {
            const int w = b0 + (tl >> lgp);
            const bool on = w < cnt;
            const int j = on ? G.flev_steps[beg + w] : 0;
            double D = 0.0, yr = 0.0;  // component c of D_j, row r of y_j
            if (on && gl == 0) {
                D = comp(&fac[j]);
                yr = r ? ys[j].y : ys[j].x;
            }
            if (on)
                for (int q = G.dg_ptr[j] + gl; q < G.dg_ptr[j + 1]; q += gs) {
                    const int p = G.dg_pos[q], k = G.dg_k[q];
                    const double lt = comp(&Lv[p]), dk = comp(&dinv[k]), u = comp(&Uv[p]);
                    double d0, d1, l0, l1;
                    const double tk = qmul(dk, u, d0, d1);  // (D_k^-1 U(k,j))_c
                    D -= qmul(lt, tk, l0, l1);              // (Lt(j,k) D_k^-1 U(k,j))_c
                    const double2 z = zs[k];
                    yr -= __fma_rn(l0, z.x, l1 * z.y);      // (Lt(j,k) z_k)_r
                }
            for (int o = gs >> 1; o > 0; o >>= 1) {
                D += __shfl_xor_sync(0xffffffffu, D, 4 * o);
                yr += __shfl_xor_sync(0xffffffffu, yr, 4 * o);
            }
            if (on && gl == 0) {
                const double Dx = __shfl_sync(qm, D, qb), Dy = __shfl_sync(qm, D, qb + 1);
                const double Dz = __shfl_sync(qm, D, qb + 2), Dw = __shfl_sync(qm, D, qb + 3);
                const double det = Dx * Dw - Dy * Dz;
                sing |= (det == 0.0 || !isfinite(det));
                const double rd = rcp_rn(det);
                const double inv = c == 0 ? Dw * rd : c == 1 ? -Dy * rd : c == 2 ? -Dz * rd : Dx * rd;
                ((double *)&dinv[j])[c] = inv;
                const double y0 = __shfl_sync(qm, yr, qb), y1 = __shfl_sync(qm, yr, qb + 2);
                const double i0 = __shfl_sync(qm, inv, sA0), i1 = __shfl_sync(qm, inv, sA1);
                if (s == 0) {
                    ((double *)&ys[j])[r] = yr;
                    ((double *)&zs[j])[r] = __fma_rn(i0, y0, i1 * y1);  // (D_j^-1 y_j)_r
                }
            }
        }
    }
    {
        // rot is a multiple of 32, so a thread keeps its lane (and quad)
        const int te = (t + rot) & (NT - 1);
        const int tl = te >> 2, gs = 1 << lge, gl = tl & (gs - 1), ng = (NT >> 2) >> lge;
        const int beg = G.fent_ptr[l], cnt = G.fent_ptr[l + 1] - beg;
        for (int b0 = 0; b0 < cnt; b0 += ng) {
            const int e = b0 + (tl >> lge);
            const bool on = e < cnt;
            const int p = on ? G.fent_p[beg + e] : 0;
            double aL = 0.0, aU = 0.0;
            if (on && gl == 0) { aL = comp(&Lv[p]); aU = comp(&Uv[p]); }
            if (on)
                for (int q = G.og_ptr[p] + gl; q < G.og_ptr[p + 1]; q += gs) {
                    const int x = G.og_a[q], y = G.og_b[q];
                    const double dk = comp(&dinv[G.og_k[q]]);
                    const double ly = comp(&Lv[y]), ux = comp(&Uv[x]), lx = comp(&Lv[x]), uy = comp(&Uv[y]);
                    double a0, a1;
                    aL -= qmul(ly, qmul(dk, ux, a0, a1), a0, a1);
                    aU -= qmul(lx, qmul(dk, uy, a0, a1), a0, a1);
                }
            for (int o = gs >> 1; o > 0; o >>= 1) {
                aL += __shfl_xor_sync(0xffffffffu, aL, 4 * o);
                aU += __shfl_xor_sync(0xffffffffu, aU, 4 * o);
            }
            if (on && gl == 0) {
                ((double *)&Uv[p])[c] = aU;
                ((double *)&Lv[p])[c] = aL;
            }
        }
    }
    return sing;
}

// The two passes of FP64 forward level l (lu_pivots, lu_entries) with each
// 2x2 block spread over a quad of four lanes, as lu_level1_q: L scaled, so a
// gather element is one block product, D_j = A_jj - sum L(j,k) U(k,j),
// y_j -= L(j,k) y_k, then U(j,i) and L(i,j) = (A_ij - sum L(i,k) U(k,j)) D_j^-1.
template <int NT>
__device__ __forceinline__ bool lu_pivots_q(const TopoView &G, int l, int lg, int t, double4_32a *fac,
                                            double4_32a *dinv, double2 *ys, const double4_32a *Lv,
                                            const double4_32a *Uv) {
    const int c = t & 3, r = c >> 1, s = c & 1, qb = (t & 31) & ~3;
    const unsigned qm = 0xfu << qb;
    const int sA0 = qb + 2 * r, sA1 = sA0 + 1, sB0 = qb + s, sB1 = qb + 2 + s;
    auto comp = [&](const double4_32a *p) { return ((const double *)p)[c]; };
    const int tl = t >> 2, gs = 1 << lg, gl = tl & (gs - 1), ng = (NT >> 2) >> lg;
    const int beg = G.flev_ptr[l], cnt = G.flev_ptr[l + 1] - beg;
    bool sing = false;
    for (int b0 = 0; b0 < cnt; b0 += ng) {
        const int w = b0 + (tl >> lg);
        const bool on = w < cnt;
        const int j = on ? G.flev_steps[beg + w] : 0;
        double D = 0.0, yr = 0.0;
        if (on && gl == 0) {
            D = comp(&fac[j]);
            yr = r ? ys[j].y : ys[j].x;
        }
        if (on)
            for (int q = G.dg_ptr[j] + gl; q < G.dg_ptr[j + 1]; q += gs) {
                const int p = G.dg_pos[q];
                const double lj = comp(&Lv[p]), u = comp(&Uv[p]);
                const double l0 = __shfl_sync(qm, lj, sA0), l1 = __shfl_sync(qm, lj, sA1);
                const double u0 = __shfl_sync(qm, u, sB0), u1 = __shfl_sync(qm, u, sB1);
                D -= __fma_rn(l0, u0, l1 * u1);             // (L(j,k) U(k,j))_c
                const double2 yk = ys[G.dg_k[q]];
                yr -= __fma_rn(l0, yk.x, l1 * yk.y);        // (L(j,k) y_k)_r
            }
        for (int o = gs >> 1; o > 0; o >>= 1) {
            D += __shfl_xor_sync(0xffffffffu, D, 4 * o);
            yr += __shfl_xor_sync(0xffffffffu, yr, 4 * o);
        }
        if (on && gl == 0) {
            const double Dx = __shfl_sync(qm, D, qb), Dy = __shfl_sync(qm, D, qb + 1);
            const double Dz = __shfl_sync(qm, D, qb + 2), Dw = __shfl_sync(qm, D, qb + 3);
            const double det = Dx * Dw - Dy * Dz;
            sing |= (det == 0.0 || !isfinite(det));
            const double rd = rcp_rn(det);
            ((double *)&dinv[j])[c] = c == 0 ? Dw * rd : c == 1 ? -Dy * rd : c == 2 ? -Dz * rd : Dx * rd;
            if (s == 0) ((double *)&ys[j])[r] = yr;
        }
    }
    return sing;
}

template <int NT>
__device__ __forceinline__ void lu_entries_q(const TopoView &G, int l, int lg, int t, const double4_32a *dinv,
                                             double4_32a *Lv, double4_32a *Uv) {
    const int c = t & 3, r = c >> 1, s = c & 1, qb = (t & 31) & ~3;
    const unsigned qm = 0xfu << qb;
    const int sA0 = qb + 2 * r, sA1 = sA0 + 1, sB0 = qb + s, sB1 = qb + 2 + s;
    auto comp = [&](const double4_32a *p) { return ((const double *)p)[c]; };
    auto qmul = [&](double a, double b) {
        const double a0 = __shfl_sync(qm, a, sA0), a1 = __shfl_sync(qm, a, sA1);
        const double b0 = __shfl_sync(qm, b, sB0), b1 = __shfl_sync(qm, b, sB1);
        return __fma_rn(a0, b0, a1 * b1);
    };
    const int tl = t >> 2, gs = 1 << lg, gl = tl & (gs - 1), ng = (NT >> 2) >> lg;
    const int beg = G.fent_ptr[l], cnt = G.fent_ptr[l + 1] - beg;
    for (int b0 = 0; b0 < cnt; b0 += ng) {
        const int e = b0 + (tl >> lg);
        const bool on = e < cnt;
        const int p = on ? G.fent_p[beg + e] : 0, j = on ? G.fent_j[beg + e] : 0;
        double aL = 0.0, aU = 0.0;
        if (on && gl == 0) { aL = comp(&Lv[p]); aU = comp(&Uv[p]); }
        if (on)
            for (int q = G.og_ptr[p] + gl; q < G.og_ptr[p + 1]; q += gs) {
                const int x = G.og_a[q], y = G.og_b[q];
                aL -= qmul(comp(&Lv[y]), comp(&Uv[x]));
                aU -= qmul(comp(&Lv[x]), comp(&Uv[y]));
            }
        for (int o = gs >> 1; o > 0; o >>= 1) {
            aL += __shfl_xor_sync(0xffffffffu, aL, 4 * o);
            aU += __shfl_xor_sync(0xffffffffu, aU, 4 * o);
        }
        if (on && gl == 0) {
            ((double *)&Uv[p])[c] = aU;
            ((double *)&Lv[p])[c] = qmul(aL, comp(&dinv[j]));  // (... D_j^-1)_c
        }
    }
}

// Forward substitution alone on FP64 level l with the quads of lu_pivots_q:
// y_j -= sum_k L(j,k) y_k summed exactly as lu_pivots_q's y part (same
// quads, groups and order), so an instance on a factor made by the quad
// pivots gets the y the fused pass would have given.
template <int NT>
__device__ __forceinline__ void fwd_rows_q(const TopoView &G, int l, int lg, int t, const double4_32a *Lv,
                                           double2 *ys) {
    const int c = t & 3, r = c >> 1, s = c & 1, qb = (t & 31) & ~3;
    const unsigned qm = 0xfu << qb;
    const int sA0 = qb + 2 * r, sA1 = sA0 + 1;
    const int tl = t >> 2, gs = 1 << lg, gl = tl & (gs - 1), ng = (NT >> 2) >> lg;
    const int beg = G.flev_ptr[l], cnt = G.flev_ptr[l + 1] - beg;
    for (int b0 = 0; b0 < cnt; b0 += ng) {
        const int w = b0 + (tl >> lg);
        const bool on = w < cnt;
        const int j = on ? G.flev_steps[beg + w] : 0;
        double yr = 0.0;
        if (on && gl == 0) yr = r ? ys[j].y : ys[j].x;
        if (on)
            for (int q = G.dg_ptr[j] + gl; q < G.dg_ptr[j + 1]; q += gs) {
                const double lj = ((const double *)&Lv[G.dg_pos[q]])[c];
                const double l0 = __shfl_sync(qm, lj, sA0), l1 = __shfl_sync(qm, lj, sA1);
                const double2 yk = ys[G.dg_k[q]];
                yr -= __fma_rn(l0, yk.x, l1 * yk.y);
            }
        for (int o = gs >> 1; o > 0; o >>= 1) yr += __shfl_xor_sync(0xffffffffu, yr, 4 * o);
        if (on && gl == 0 && s == 0) ((double *)&ys[j])[r] = yr;
    }
}

// fwd_rows on 32 lanes for a factor made by lu_two_pass_warp: the quads'
// order on the levels that took them, else one lane a row.
template <typename TJ>
__device__ __forceinline__ void fwd_rows_warp(const TopoView &G, int l, bool grouped, bool quad, int lane,
                                              const typename Blk<TJ>::b4 *Lv, typename Blk<TJ>::b2 *ys) {
    if constexpr (sizeof(TJ) == 8) {
        if (quad && G.lvl_q4w[l]) {
            fwd_rows_q<32>(G, l, grouped ? G.lvl_group4w[2 * l] : 0, lane, Lv, ys);
            return;
        }
    }
    fwd_rows<TJ, 32>(G, l, grouped ? G.lvl_group_w[3 * l] : 0, lane, Lv, ys);
}

// Two-pass forward level l on 32 lanes (the warp kernel, the shared flat
// start, a block's narrow levels): FP64 levels that fit the warp's eight
// quads (lvl_q4w) take lu_pivots_q / lu_entries_q, the rest one lane a block.
// grouped = 0 gives every pivot and entry one lane (quad) of its own.
template <typename TJ>
__device__ __forceinline__ bool lu_two_pass_warp(const TopoView &G, int l, bool grouped, bool quad, int lane,
                                                 typename Blk<TJ>::b4 *fac, typename Blk<TJ>::b4 *dinv,
                                                 typename Blk<TJ>::b2 *ys, typename Blk<TJ>::b4 *Lv,
                                                 typename Blk<TJ>::b4 *Uv) {
    if constexpr (sizeof(TJ) == 8) {
        if (quad && G.lvl_q4w[l]) {
            const bool sing = lu_pivots_q<32>(G, l, grouped ? G.lvl_group4w[2 * l] : 0, lane, fac, dinv, ys, Lv, Uv);
            __syncwarp();
            lu_entries_q<32>(G, l, grouped ? G.lvl_group4w[2 * l + 1] : 0, lane, dinv, Lv, Uv);
            return sing;
        }
    }
    const bool sing = lu_pivots<TJ, 32>(G, l, grouped ? G.lvl_group_w[3 * l] : 0, lane, fac, dinv, ys, Lv, Uv);
    __syncwarp();
    lu_entries<TJ, 32>(G, l, grouped ? G.lvl_group_w[3 * l + 1] : 0, lane, dinv, Lv, Uv);
    return sing;
}

// GS: the state placement level of layout(); 3 = level 2 compiled for four
// blocks per SM (64 registers a thread) instead of two.
template <typename TJ, int GS>
__global__ void __launch_bounds__(kThreads, GS == 3 ? 4 : 2) k_nr_block(Args a) {
    constexpr int LV = GS > 2 ? 2 : GS;
    using B4 = typename Blk<TJ>::b4;
    using B2 = typename Blk<TJ>::b2;
    extern __shared__ __align__(32) unsigned char smem[];
    __shared__ unsigned long long red[kWarps];
    __shared__ int s_inst, s_done, s_status, s_it, s_nev, s_topo, s_wcnt[kWarps];
    __shared__ double s_maxG, s_maxDx;
    const unsigned long long tol_bits = abits(a.tol), tol10_bits = abits(a.tol * 10.);
    const bool keep_cs = sizeof(TJ) == 8 || a.rotate;  // who reads the FP64 cos, sin
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned char *ism = smem + a.blob_region;  // per-instance region
    if (tid == 0) s_topo = -1;
    for (;;) {
        if (tid == 0) {
            const int q = atomicAdd(a.counter, 1);
            const int qlen = a.resume ? *a.handoff_n : a.queue_len;
            s_inst = q < qlen ? a.queue[q] : -1;
        }
        __syncthreads();
        const int inst = s_inst;
        if (inst < 0) break;
        const int t_id = a.inst_topo[inst];
        const Topo T = a.topo[t_id];
        // stage the topology's blob in shared memory unless it is already there
        const char *blob = T.blob;
        if (T.blob_smem) {
            if (s_topo != t_id) {
                const int4 *src = (const int4 *)T.blob;
                int4 *dst = (int4 *)smem;
                for (int i = tid; i < T.blob_bytes / 16; i += kThreads) dst[i] = src[i];
                __syncthreads();
                if (tid == 0) s_topo = t_id;
            }
            blob = (const char *)smem;
        }
        const TopoView G = bind(T.o, blob);
        const long long off = a.inst_off[inst];
        const Layout L = layout<TJ>(T.nB, T.n, T.nup, T.nPV, T.fac_smem, a.lu1, LV);
        // the state arrays layout() moves to global memory (LV)
        unsigned char *gst = LV ? a.gstate + (long long)blockIdx.x * a.gstate_stride : ism;
        unsigned char *vst = (LV >= 2 || (LV && sizeof(TJ) == 4)) ? gst : ism;
        unsigned char *pst = LV >= 2 ? gst : ism;  // phasors
        double *V = (double *)(vst + L.V), *th = (double *)(gst + L.th);
        double *cs = (double *)(vst + L.cs), *sn = (double *)(vst + L.sn);
        double2 *ef = (double2 *)(pst + L.ef);
        float4 *f32 = (float4 *)(pst + L.f32);
        double *P = (double *)(gst + L.P), *Q = (double *)(gst + L.Q), *QL = (double *)(gst + L.QL);
        unsigned char *act = ism + L.act;
        int *limQ = (int *)(ism + L.lim);
        B2 *ys = (B2 *)(ism + L.ys);
        // the inverse of each diagonal block overwrites it (dinv = fac)
        B4 *fac = T.fac_smem ? (B4 *)(ism + L.fac) : (B4 *)(a.scratch + (long long)blockIdx.x * a.scratch_stride);
        B4 *dinv = fac;
        const int n = T.n, nB = T.nB, nq = T.n + 2 * T.nup;
        B4 *Lv = fac + n, *Uv = fac + n + T.nup;
        int wk = a.kind ? a.kind[inst] : 0;
        bool from_park = a.resume;
        // a failed run from a predicted start runs again from the own start
        for (;;) {
            const bool pred = wk == 1;
            const int mi = pred ? a.warm_max_iter : a.max_iter;
            if (!from_park) {
                // initLim (GPU/limiteInjReat.cuh:188-224) and the starting state
                const double *v0 = pred ? a.Vp : a.V0, *t0 = pred ? a.thp : a.th0;
                for (int k = tid; k < nB; k += kThreads) {
                    V[k] = v0[off + k];
                    th[k] = t0[off + k];
                    QL[k] = a.Qliq[off + k];
                    act[k] = (G.type[k] == 0 || G.type[k] == 1);
                }
                for (int i = tid; i < T.nPV; i += kThreads) limQ[i] = 0;
                if (a.trig)
                    for (int k = tid; k < a.hist_cap; k += kThreads) a.trig[k] = 0;
                if (tid == 0) { s_done = 0; s_status = 0; s_it = 0; s_nev = 0; s_maxDx = INFINITY; }
            } else {
                // the state a warp parked at the hand-off
                for (int k = tid; k < nB; k += kThreads) {
                    V[k] = a.V[off + k];
                    th[k] = a.th[off + k];
                    QL[k] = a.Q[off + k];
                    act[k] = (G.type[k] == 0 || G.type[k] == 1);
                }
                __syncthreads();
                for (int i = tid; i < T.nPV; i += kThreads) {
                    limQ[i] = (int)a.P[off + i];
                    act[G.pv_bus[i]] = limQ[i];
                }
                if (tid == 0) {
                    s_done = 0; s_status = 0;
                    s_it = a.iters[inst]; s_nev = a.n_events[inst]; s_maxDx = a.mism[inst];
                }
            }
            __syncthreads();
            bool fresh = true;
            // iteration 0 from the grid's own start: the topology's shared copy
            const char *flat = (!from_park && !pred && T.flat && a.flat_on && *a.flat_on) ? T.flat : nullptr;
            const FlatLayout F = flat_layout<TJ>(nB, nq);
            // iteration 0 from a predicted start: the reference factor, unless singular
            const char *wref = (!from_park && pred && a.wref && !*(const int *)(a.wref + F.sing)) ? a.wref : nullptr;
            for (;;) {
                const bool f0 = flat && s_it == 0;
                const bool c0 = wref && s_it == 0;
                if (f0) {
                    for (int k = tid; k < nB; k += kThreads) {
                        if (keep_cs) {
                            cs[k] = ((const double *)(flat + F.cs))[k];
                            sn[k] = ((const double *)(flat + F.sn))[k];
                        }
                        ef[k] = ((const double2 *)(flat + F.ef))[k];
                        if (sizeof(TJ) == 4) f32[k] = ((const float4 *)(flat + F.f32))[k];
                        P[k] = ((const double *)(flat + F.P))[k];
                        Q[k] = ((const double *)(flat + F.Q))[k];
                    }
                } else {
                    // phasors (the FP32-LU form may rotate them in the update
                    // instead) and injections
                    if (sizeof(TJ) == 8 || fresh || !a.rotate)
                        for (int k = tid; k < nB; k += kThreads) phasor<TJ>(k, th, V, cs, sn, ef, f32, keep_cs);
                    __syncthreads();
                    for (int i = tid; i < nB; i += kThreads) {
                        const int k = G.inj_order[i];
                        injection(G.yptr, G.ycol, G.yval, ef, k, P[k], Q[k]);
                    }
                }
                fresh = false;
                __syncthreads();
                const int it = s_it;
                // reactive limits (chkLimQ) when the previous step was small
                if (a.lim && it >= 1 && it < mi && abits(s_maxDx) < tol10_bits) {
                    if (a.trig && tid == 0 && it < a.hist_cap) a.trig[it] = 1;
                    for (int i0 = 0; i0 < T.nPV; i0 += kThreads) {
                        const int i = i0 + tid;
                        int code = 0, b = 0;
                        if (i < T.nPV) {
                            b = G.pv_bus[i];
                            const double ql = a.Qload[off + b], qg = Q[b] + ql;
                            if (qg < G.Qmin[i] - a.tol) {
                                if (!limQ[i]) code = 1;
                                else if (QL[b] != G.Qmin[i] - ql) code = 2;
                                limQ[i] = 1;
                                QL[b] = G.Qmin[i] - ql;
                            } else if (qg > G.Qmax[i] + a.tol) {
                                if (!limQ[i]) code = 3;
                                else if (QL[b] != G.Qmax[i] - ql) code = 4;
                                limQ[i] = 1;
                                QL[b] = G.Qmax[i] - ql;
                            } else {
                                if (limQ[i]) code = 5;
                                limQ[i] = 0;
                            }
                            act[b] = limQ[i];
                        }
                        // events in PV order, as chkLimQ prints them: a
                        // block-wide exclusive count of the events before i
                        const unsigned m = __ballot_sync(0xffffffffu, code != 0);
                        if (lane == 0) s_wcnt[warp] = __popc(m);
                        __syncthreads();
                        int e = s_nev + __popc(m & ((1u << lane) - 1u)), tot = 0;
                        for (int w = 0; w < kWarps; w++) {
                            if (w < warp) e += s_wcnt[w];
                            tot += s_wcnt[w];
                        }
                        if (code && e < a.ev_cap) {
                            int *ev = a.events + ((long long)inst * a.ev_cap + e) * 4;
                            ev[0] = it; ev[1] = b + 1; ev[2] = i; ev[3] = code;
                        }
                        __syncthreads();
                        if (tid == 0) s_nev += tot;
                    }
                    __syncthreads();
                }
                // mismatch (FP64) and convergence test
                unsigned long long m = 0;
                for (int j = tid; j < n; j += kThreads) {
                    const int k = G.bus_of_blk[j];
                    const double gp = a.Pliq[off + k] - P[k];
                    const double gq = act[k] ? QL[k] - Q[k] : 0.0;
                    B2 r;
                    r.x = (TJ)gp;
                    r.y = (TJ)gq;
                    ys[j] = r;
                    m = umax64(m, umax64(abits(gp), abits(gq)));
                }
                m = block_umax(m, red);
                if (tid == 0) {
                    s_maxG = __longlong_as_double((long long)m);
                    if (a.hist && it < a.hist_cap) a.hist[it] = s_maxG;
                    if (m > kInfBits) { s_status = GBPF_E_NOCONV; s_done = 1; }
                    else if (m <= tol_bits) s_done = 1;
                    else if (it >= mi) { s_status = GBPF_E_NOCONV; s_done = 1; }
                }
                __syncthreads();
                if (s_done) break;
                const B4 *Ub = Uv, *Db = dinv;
                if (f0 || c0) {
                    // a shared factor (the grid's start, or the warm start's
                    // reference): forward substitution alone
                    const char *sb = f0 ? flat : wref;
                    const B4 *facS = (const B4 *)(sb + F.fac);
                    if (*(const int *)(sb + F.sing)) {
                        if (tid == 0) { s_status = GBPF_E_SINGULAR; s_done = 1; }
                        __syncthreads();
                        break;
                    }
                    for (int l = 0; l < T.nfl; l++) {
                        fwd_rows<TJ, kThreads>(G, l, a.no_group ? 0 : G.lvl_group[3 * l], tid, facS + n, ys);
                        __syncthreads();
                    }
                    Ub = facS + n + T.nup;
                    Db = facS;
                } else {
                    // Jacobian fill at every factor position (zeros at fill-in)
                    for (int q = tid; q < nq; q += kThreads) fac[q] = jac_block<TJ>(G, q, n, act, P, Q, V, cs, sn, f32);
                    __syncthreads();
                    // LU factorisation fused with forward substitution, one level at a
                    // time, in two passes: pivots (diagonal block, its inverse, y_j),
                    // then the level's off-diagonal entries.  A level narrow enough
                    // for one warp (lvl_narrow) runs on warp 0 alone with warp
                    // syncs, lanes grouped by lvl_group_w, and the block meets at a
                    // barrier only where a wide level follows; wide levels use the
                    // whole block, lanes grouped by lvl_group.
                    // With lu1 each level is one pass (lu_level1: pivots and entries
                    // side by side, L unscaled) and needs one barrier instead of two.
                    B2 *zs = (B2 *)(ism + L.zs);
                    for (int l = 0; l < T.nfl; l++) {
                        if (a.narrow && (G.lvl_narrow[l] & 1)) {
                            if (warp == 0) {
                                const int gp = a.no_group ? 0 : G.lvl_group_w[3 * l];
                                const int ge = a.no_group ? 0 : G.lvl_group_w[3 * l + 1];
                                bool sing;
                                if (a.lu1) {
                                    sing = lu_level1<TJ, 32>(G, l, gp, ge, a.no_group ? 0 : G.lvl_rot[l] >> 16, lane,
                                                             fac, dinv, ys, zs, Lv, Uv);
                                } else {
                                    sing = lu_two_pass_warp<TJ>(G, l, !a.no_group, a.quad, lane, fac, dinv, ys, Lv, Uv);
                                }
                                if (sing) { s_status = GBPF_E_SINGULAR; s_done = 1; }
                                __syncwarp();
                            }
                            if (l + 1 == T.nfl || !(G.lvl_narrow[l + 1] & 1)) __syncthreads();
                        } else {
                            const int gp = a.no_group ? 0 : G.lvl_group[3 * l];
                            const int ge = a.no_group ? 0 : G.lvl_group[3 * l + 1];
                            if (a.lu1) {
                                bool sing;
                                if constexpr (sizeof(TJ) == 8) {
                                    if (a.quad && G.lvl_rot4[l] >= 0) {
                                        sing = lu_level1_q<kThreads>(
                                            G, l, a.no_group ? 0 : G.lvl_group4[2 * l],
                                            a.no_group ? 0 : G.lvl_group4[2 * l + 1], a.no_group ? 0 : G.lvl_rot4[l],
                                            tid, fac, dinv, ys, zs, Lv, Uv);
                                    } else {
                                        sing = lu_level1<TJ, kThreads>(G, l, gp, ge,
                                                                       a.no_group ? 0 : G.lvl_rot[l] & 0xffff, tid,
                                                                       fac, dinv, ys, zs, Lv, Uv);
                                    }
                                } else {
                                    sing = lu_level1<TJ, kThreads>(G, l, gp, ge, a.no_group ? 0 : G.lvl_rot[l] & 0xffff,
                                                                   tid, fac, dinv, ys, zs, Lv, Uv);
                                }
                                if (sing) { s_status = GBPF_E_SINGULAR; s_done = 1; }
                            } else {
                                bool q4 = false;
                                if constexpr (sizeof(TJ) == 8) q4 = a.quad && G.lvl_rot4[l] >= 0;
                                if (q4) {
                                    if constexpr (sizeof(TJ) == 8) {
                                        const int gp4 = a.no_group ? 0 : G.lvl_group4[2 * l];
                                        const int ge4 = a.no_group ? 0 : G.lvl_group4[2 * l + 1];
                                        const bool sing = lu_pivots_q<kThreads>(G, l, gp4, tid, fac, dinv, ys, Lv, Uv);
                                        if (sing) { s_status = GBPF_E_SINGULAR; s_done = 1; }
                                        __syncthreads();
                                        lu_entries_q<kThreads>(G, l, ge4, tid, dinv, Lv, Uv);
                                    }
                                } else {
                                    const bool sing = lu_pivots<TJ, kThreads>(G, l, gp, tid, fac, dinv, ys, Lv, Uv);
                                    if (sing) { s_status = GBPF_E_SINGULAR; s_done = 1; }
                                    __syncthreads();
                                    lu_entries<TJ, kThreads>(G, l, ge, tid, dinv, Lv, Uv);
                                }
                            }
                            __syncthreads();
                        }
                    }
                }
                if (s_done) break;
                // backward substitution, level by level, narrow levels on warp 0
                for (int l = 0; l < T.nbl; l++) {
                    if (a.narrow && (G.lvl_narrow[l] & 2)) {
                        if (warp == 0) {
                            back_rows<TJ, 32>(G, l, a.no_group ? 0 : G.lvl_group_w[3 * l + 2], lane, Db, Ub, ys);
                            __syncwarp();
                        }
                        if (l + 1 == T.nbl || !(G.lvl_narrow[l + 1] & 2)) __syncthreads();
                    } else {
                        back_rows<TJ, kThreads>(G, l, a.no_group ? 0 : G.lvl_group[3 * l + 2], tid, Db, Ub, ys);
                        __syncthreads();
                    }
                }
                // update (FP64 state) and max|dx|
                unsigned long long md = 0;
                for (int j = tid; j < n; j += kThreads) {
                    const int k = G.bus_of_blk[j];
                    const double dt = (double)ys[j].x, dv = (double)ys[j].y;
                    th[k] += dt;
                    if (act[k]) V[k] += dv;
                    if (sizeof(TJ) == 4 && a.rotate) {
                        double c = cs[k], s = sn[k];
                        rotate_phasor(th[k], dt, c, s);
                        cs[k] = c;
                        sn[k] = s;
                        ef[k] = make_double2(V[k] * c, V[k] * s);
                        f32[k] = make_float4((float)c, (float)s, (float)V[k], 0.f);
                    }
                    md = umax64(md, umax64(abits(dt), abits(dv)));
                }
                md = block_umax(md, red);
                if (tid == 0) { s_maxDx = __longlong_as_double((long long)md); s_it = it + 1; }
                __syncthreads();
            }
            if (!pred) break;
            // the predicted run: kept, or started again from the own start
            unsigned long long dv = 0;
            for (int k = tid; k < nB; k += kThreads)
                if (G.type[k] == 0 || G.type[k] == 1) dv = umax64(dv, abits(V[k] - a.Vp[off + k]));
            dv = block_umax(dv, red);
            const bool fail = s_status != 0 || dv > abits(a.warm_max_dv);
            if (tid == 0) {
                a.witers[inst] = s_it;
                if (fail) a.kind[inst] = 2;
            }
            __syncthreads();
            if (!fail) break;
            wk = 2;
            from_park = false;
        }
        // results
        for (int k = tid; k < nB; k += kThreads) {
            a.V[off + k] = V[k];
            a.th[off + k] = th[k];
            a.P[off + k] = P[k];
            a.Q[off + k] = Q[k];
        }
        if (tid == 0) {
            a.iters[inst] = s_it;
            a.status[inst] = s_status;
            a.mism[inst] = s_maxG;
            a.n_events[inst] = s_nev;
        }
        if (a.limq_out)
            for (int i = tid; i < T.nPV; i += kThreads) a.limq_out[i] = limQ[i];
        if (a.ctl_out && tid == 0) {
            gbpf::SolveCtl c{};
            c.it = s_it;
            c.done = 1;
            c.status = s_status;
            c.n_events = s_nev;
            c.maxG = (unsigned long long)__double_as_longlong(s_maxG);
            c.maxDx = (unsigned long long)__double_as_longlong(s_maxDx);
            c.converged = s_status == 0;
            *a.ctl_out = c;
        }
        __syncthreads();
    }
}


// One instance per warp: the same Newton loop as k_nr_block with the 32 lanes
// of a warp in place of the threads of a block, so the only barriers are
// __syncwarp.  Each warp owns a slice of the block's dynamic shared memory
// (state and factor); the topology's read-only blob is read from global
// memory through the L1 cache.
// Iteration 0 of every instance of topology T that starts from the grid's
// own state (FlatLayout): one warp, the warp kernel's own arithmetic (same
// functions, lane groups and order), so an instance that takes it gets the
// values it would have computed itself.  Shared memory: ys (zero right-hand
// side; only the factor is kept) and the active-voltage flags.
template <typename TJ>
__global__ void __launch_bounds__(32) k_flat_start(const Topo T, char *out, int warp_group, int quad) {
    using B4 = typename Blk<TJ>::b4;
    using B2 = typename Blk<TJ>::b2;
    extern __shared__ __align__(16) unsigned char fsm[];
    const int lane = threadIdx.x;
    const TopoView G = bind(T.o, T.blob);
    const int n = T.n, nB = T.nB, nq = T.n + 2 * T.nup;
    const FlatLayout F = flat_layout<TJ>(nB, nq);
    const double *V = (const double *)(out + F.V0), *th = (const double *)(out + F.th0);
    double *cs = (double *)(out + F.cs), *sn = (double *)(out + F.sn), *P = (double *)(out + F.P),
           *Q = (double *)(out + F.Q);
    double2 *ef = (double2 *)(out + F.ef);
    float4 *f32 = (float4 *)(out + F.f32);
    B4 *fac = (B4 *)(out + F.fac), *Lv = fac + n, *Uv = fac + n + T.nup;
    B2 *ys = (B2 *)fsm;
    unsigned char *act = fsm + align_up(sizeof(B2) * n, 16);
    for (int k = lane; k < nB; k += 32) {
        phasor<TJ>(k, th, V, cs, sn, ef, f32);
        act[k] = (G.type[k] == 0 || G.type[k] == 1);
    }
    for (int j = lane; j < n; j += 32) ys[j].x = ys[j].y = (TJ)0;
    __syncwarp();
    for (int i = lane; i < nB; i += 32) {
        const int k = G.inj_order[i];
        injection(G.yptr, G.ycol, G.yval, ef, k, P[k], Q[k]);
    }
    __syncwarp();
    for (int q = lane; q < nq; q += 32) fac[q] = jac_block<TJ>(G, q, n, act, P, Q, V, cs, sn, f32);
    __syncwarp();
    bool sing = false;
    for (int l = 0; l < T.nfl; l++) {
        sing |= lu_two_pass_warp<TJ>(G, l, warp_group != 0, quad != 0, lane, fac, fac, ys, Lv, Uv);
        __syncwarp();
    }
    sing = __any_sync(0xffffffffu, sing);
    if (lane == 0) *(int *)(out + F.sing) = sing ? 1 : 0;
}

// GS: the state placement level of layout() (the region of warp w of block b
// starts at gstate + (b * warps per block + w) * gstate_stride); 3 = level 2
// compiled for two blocks of 16 warps per SM (64 registers a thread).
template <typename TJ, int GS>
__global__ void __launch_bounds__(32 * kWarpsMax, GS == 3 ? 2 : 1) k_nr_warp(Args a) {
    constexpr int LV = GS > 2 ? 2 : GS;
    using B4 = typename Blk<TJ>::b4;
    using B2 = typename Blk<TJ>::b2;
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ __align__(32) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    unsigned char *ism = smem + (size_t)(threadIdx.x >> 5) * a.slice;
    const unsigned lt_mask = (1u << lane) - 1u;
    const unsigned long long tol_bits = abits(a.tol), tol10_bits = abits(a.tol * 10.);
    const bool keep_cs = sizeof(TJ) == 8 || a.rotate;  // who reads the FP64 cos, sin
    for (;;) {
        int q = 0;
        if (lane == 0) q = atomicAdd(a.counter, 1);
        q = __shfl_sync(FULL, q, 0);
        if (q >= a.queue_len) break;
        const int inst = a.queue[q];
        const int t_id = a.inst_topo[inst];
        const Topo T = a.topo[t_id];
        const TopoView G = bind(T.o, T.blob);
        const long long off = a.inst_off[inst];
        const Layout L = layout<TJ>(T.nB, T.n, T.nup, T.nPV, 1, a.lu1, LV);
        unsigned char *gst =
            LV ? a.gstate + ((long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * a.gstate_stride : ism;
        unsigned char *vst = (LV >= 2 || (LV && sizeof(TJ) == 4)) ? gst : ism;
        unsigned char *pst = LV >= 2 ? gst : ism;  // phasors
        double *V = (double *)(vst + L.V), *th = (double *)(gst + L.th);
        double *cs = (double *)(vst + L.cs), *sn = (double *)(vst + L.sn);
        double2 *ef = (double2 *)(pst + L.ef);
        float4 *f32 = (float4 *)(pst + L.f32);
        double *P = (double *)(gst + L.P), *Q = (double *)(gst + L.Q), *QL = (double *)(gst + L.QL);
        unsigned char *act = ism + L.act;
        int *limQ = (int *)(ism + L.lim);
        B2 *ys = (B2 *)(ism + L.ys);
        B4 *fac = (B4 *)(ism + L.fac), *dinv = fac;  // block inverses overwrite the diagonal
        const int n = T.n, nB = T.nB, nq = T.n + 2 * T.nup;
        B4 *Lv = fac + n, *Uv = fac + n + T.nup;
        const FlatLayout F = flat_layout<TJ>(nB, nq);
        int wk = a.kind ? a.kind[inst] : 0;
        int it, status, nev;
        double maxDx, maxG;
        bool parked;
        // a failed run from a predicted start runs again from the own start
        for (;;) {
            const bool pred = wk == 1;
            const int mi = pred ? a.warm_max_iter : a.max_iter;
            const char *flat = (!pred && T.flat && a.flat_on && *a.flat_on) ? T.flat : nullptr;
            // iteration 0 from a predicted start: the reference factor, unless singular
            const char *wref = (pred && a.wref && !*(const int *)(a.wref + F.sing)) ? a.wref : nullptr;
            const double *v0 = pred ? a.Vp : a.V0, *t0 = pred ? a.thp : a.th0;
            for (int k = lane; k < nB; k += 32) {
                V[k] = v0[off + k];
                th[k] = t0[off + k];
                QL[k] = a.Qliq[off + k];
                act[k] = (G.type[k] == 0 || G.type[k] == 1);
            }
            for (int i = lane; i < T.nPV; i += 32) limQ[i] = 0;
            it = 0, status = 0, nev = 0;
            maxDx = INFINITY, maxG = 0;
            parked = false;
            __syncwarp();
            for (;;) {
                if (a.handoff_it > 0 && it == a.handoff_it) {
                    // still iterating: park the state for the block-per-instance kernel
                    for (int k = lane; k < nB; k += 32) {
                        a.V[off + k] = V[k];
                        a.th[off + k] = th[k];
                        a.Q[off + k] = QL[k];
                    }
                    for (int i = lane; i < T.nPV; i += 32) a.P[off + i] = (double)limQ[i];
                    if (lane == 0) {
                        a.iters[inst] = it;
                        a.n_events[inst] = nev;
                        a.mism[inst] = maxDx;
                        a.handoff_q[atomicAdd(a.handoff_n, 1)] = inst;
                    }
                    parked = true;
                    break;
                }
                const bool f0 = it == 0 && flat;
                if (f0) {
                    // the shared iteration 0 of this topology's start
                    for (int k = lane; k < nB; k += 32) {
                        if (keep_cs) {
                            cs[k] = ((const double *)(flat + F.cs))[k];
                            sn[k] = ((const double *)(flat + F.sn))[k];
                        }
                        ef[k] = ((const double2 *)(flat + F.ef))[k];
                        if (sizeof(TJ) == 4) f32[k] = ((const float4 *)(flat + F.f32))[k];
                        P[k] = ((const double *)(flat + F.P))[k];
                        Q[k] = ((const double *)(flat + F.Q))[k];
                    }
                } else {
                    if (sizeof(TJ) == 8 || it == 0 || !a.rotate)
                        for (int k = lane; k < nB; k += 32) phasor<TJ>(k, th, V, cs, sn, ef, f32, keep_cs);
                    __syncwarp();
                    for (int i = lane; i < nB; i += 32) {
        const int k = G.inj_order[i];
        injection(G.yptr, G.ycol, G.yval, ef, k, P[k], Q[k]);
    }
                }
                __syncwarp();
                if (a.lim && it >= 1 && it < mi && abits(maxDx) < tol10_bits) {
                    for (int i0 = 0; i0 < T.nPV; i0 += 32) {
                        const int i = i0 + lane;
                        int code = 0, b = 0;
                        if (i < T.nPV) {
                            b = G.pv_bus[i];
                            const double ql = a.Qload[off + b], qg = Q[b] + ql;
                            if (qg < G.Qmin[i] - a.tol) {
                                if (!limQ[i]) code = 1;
                                else if (QL[b] != G.Qmin[i] - ql) code = 2;
                                limQ[i] = 1;
                                QL[b] = G.Qmin[i] - ql;
                            } else if (qg > G.Qmax[i] + a.tol) {
                                if (!limQ[i]) code = 3;
                                else if (QL[b] != G.Qmax[i] - ql) code = 4;
                                limQ[i] = 1;
                                QL[b] = G.Qmax[i] - ql;
                            } else {
                                if (limQ[i]) code = 5;
                                limQ[i] = 0;
                            }
                            act[b] = limQ[i];
                        }
                        // events in PV order, as chkLimQ prints them
                        const unsigned m = __ballot_sync(FULL, code != 0);
                        const int e = nev + __popc(m & lt_mask);
                        if (code && e < a.ev_cap) {
                            int *ev = a.events + ((long long)inst * a.ev_cap + e) * 4;
                            ev[0] = it; ev[1] = b + 1; ev[2] = i; ev[3] = code;
                        }
                        nev += __popc(m);
                    }
                    __syncwarp();
                }
                unsigned long long mloc = 0;
                for (int j = lane; j < n; j += 32) {
                    const int k = G.bus_of_blk[j];
                    const double gp = a.Pliq[off + k] - P[k];
                    const double gq = act[k] ? QL[k] - Q[k] : 0.0;
                    B2 r;
                    r.x = (TJ)gp;
                    r.y = (TJ)gq;
                    ys[j] = r;
                    mloc = umax64(mloc, umax64(abits(gp), abits(gq)));
                }
                mloc = warp_umax(mloc);
                maxG = __longlong_as_double((long long)mloc);
                if (mloc > kInfBits) { status = GBPF_E_NOCONV; break; }
                if (mloc <= tol_bits) break;
                if (it >= mi) { status = GBPF_E_NOCONV; break; }
                const B4 *Ub = Uv, *Db = dinv;
                if (f0 || (wref && it == 0)) {
                    // a shared factor (the grid's start, or the warm start's
                    // reference): forward substitution alone
                    const char *sb = f0 ? flat : wref;
                    const B4 *facS = (const B4 *)(sb + F.fac);
                    if (*(const int *)(sb + F.sing)) { status = GBPF_E_SINGULAR; break; }
                    for (int l = 0; l < T.nfl; l++) {
                        fwd_rows_warp<TJ>(G, l, a.warp_group != 0, a.quad != 0, lane, facS + n, ys);
                        __syncwarp();
                    }
                    Ub = facS + n + T.nup;
                    Db = facS;
                } else {
                    for (int qq = lane; qq < nq; qq += 32) fac[qq] = jac_block<TJ>(G, qq, n, act, P, Q, V, cs, sn, f32);
                    __syncwarp();
                    // LU fused with forward substitution, level by level, as in
                    // the block kernel with 32 lanes
                    bool sing = false;
                    B2 *zs = (B2 *)(ism + L.zs);
                    for (int l = 0; l < T.nfl; l++) {
                        const int gp = a.warp_group ? G.lvl_group_w[3 * l] : 0,
                                  ge = a.warp_group ? G.lvl_group_w[3 * l + 1] : 0;
                        if (a.lu1) {
                            sing |= lu_level1<TJ, 32>(G, l, gp, ge, a.warp_group ? G.lvl_rot[l] >> 16 : 0, lane, fac, dinv,
                                                      ys, zs, Lv, Uv);
                        } else {
                            sing |= lu_two_pass_warp<TJ>(G, l, a.warp_group != 0, a.quad != 0, lane, fac, dinv, ys, Lv,
                                                         Uv);
                        }
                        __syncwarp();
                    }
                    if (__any_sync(FULL, sing)) { status = GBPF_E_SINGULAR; break; }
                }
                for (int l = 0; l < T.nbl; l++) {
                    back_rows<TJ, 32>(G, l, a.warp_group ? G.lvl_group_w[3 * l + 2] : 0, lane, Db, Ub, ys);
                    __syncwarp();
                }
                unsigned long long md = 0;
                for (int j = lane; j < n; j += 32) {
                    const int k = G.bus_of_blk[j];
                    const double dt = (double)ys[j].x, dv = (double)ys[j].y;
                    th[k] += dt;
                    if (act[k]) V[k] += dv;
                    if (sizeof(TJ) == 4 && a.rotate) {
                        double c = cs[k], s = sn[k];
                        rotate_phasor(th[k], dt, c, s);
                        cs[k] = c;
                        sn[k] = s;
                        ef[k] = make_double2(V[k] * c, V[k] * s);
                        f32[k] = make_float4((float)c, (float)s, (float)V[k], 0.f);
                    }
                    md = umax64(md, umax64(abits(dt), abits(dv)));
                }
                maxDx = __longlong_as_double((long long)warp_umax(md));
                it++;
                __syncwarp();
            }
            __syncwarp();
            if (parked || !pred) break;
            // the predicted run: kept, or started again from the own start
            unsigned long long dv = 0;
            for (int k = lane; k < nB; k += 32)
                if (G.type[k] == 0 || G.type[k] == 1) dv = umax64(dv, abits(V[k] - a.Vp[off + k]));
            const bool fail = status != 0 || warp_umax(dv) > abits(a.warm_max_dv);
            if (lane == 0) {
                a.witers[inst] = it;
                if (fail) a.kind[inst] = 2;
            }
            __syncwarp();
            if (!fail) break;
            wk = 2;
        }
        if (parked) continue;
        for (int k = lane; k < nB; k += 32) {
            a.V[off + k] = V[k];
            a.th[off + k] = th[k];
            a.P[off + k] = P[k];
            a.Q[off + k] = Q[k];
        }
        if (lane == 0) {
            a.iters[inst] = it;
            a.status[inst] = status;
            a.mism[inst] = maxG;
            a.n_events[inst] = nev;
        }
        __syncwarp();
    }
}

__global__ void k_batch_ybus(const int *cptr, const int *csrc, const double2 *stamp, const double *gsh,
                             const double *bsh, double2 *yval, float2 *yval32, int nnz) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nnz) return;
    double2 acc = make_double2(0, 0);
    for (int c = cptr[s]; c < cptr[s + 1]; c++) {
        const int src = csrc[c];
        const double2 v = src >= 0 ? stamp[src] : make_double2(gsh[-1 - src], bsh[-1 - src]);
        if (c == cptr[s]) acc = v;
        else { acc.x += v.x; acc.y += v.y; }
    }
    yval[s] = acc;
    yval32[s] = make_float2((float)acc.x, (float)acc.y);
}

__device__ __forceinline__ double2 cdiv2(double a, double b, double c, double d) {
    if (fabs(c) >= fabs(d)) {
        const double r = d / c, den = c + d * r;
        return make_double2((a + b * r) / den, (b - a * r) / den);
    }
    const double r = c / d, den = c * r + d;
    return make_double2((a * r + b) / den, (b * r - a) / den);
}

// Branch stamps of calcYbusSp_eficinte (GPU/sistema.h:708-719) or, for a grid
// read from a .m file, calcYbusSp_Matpower (GPU/sistema.h:760-855): the
// from-side term (y + jb/2)/|t|^2 and the off-diagonals as (-1/conj(t))/z, (-1/t)/z.
__global__ void k_batch_stamps(const double *r, const double *x, const double *bch, const double *tre,
                               const double *tim, double2 *stamp, int nL, int form) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nL) return;
    const double2 y = cdiv2(1.0, 0.0, r[b], x[b]);
    double m = hypot(tre[b], tim[b]);
    m = 1.0 / (m * m);
    const double hb = bch[b] / 2.;
    if (form == GBPF_YBUS_MATPOWER) {
        const double2 uf = cdiv2(-1.0, 0.0, tre[b], -tim[b]), ut = cdiv2(-1.0, 0.0, tre[b], tim[b]);
        stamp[4 * b + 0] = cdiv2(uf.x, uf.y, r[b], x[b]);
        stamp[4 * b + 1] = cdiv2(ut.x, ut.y, r[b], x[b]);
        stamp[4 * b + 2] = make_double2(y.x * m, (y.y + hb) * m);
    } else {
        stamp[4 * b + 0] = cdiv2(-y.x, -y.y, tre[b], -tim[b]);
        stamp[4 * b + 1] = cdiv2(-y.x, -y.y, tre[b], tim[b]);
        stamp[4 * b + 2] = make_double2(m * y.x, m * y.y + hb);
    }
    stamp[4 * b + 3] = make_double2(y.x, y.y + hb);
}

#define CK(call)                                                                     \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));          \
            return GBPF_E_CUDA;                                                      \
        }                                                                            \
    } while (0)
// a kernel launch's configuration error, reported with the source line
#define CK_LAUNCH()                                                                  \
    do {                                                                             \
        cudaError_t e_ = cudaGetLastError();                                         \
        if (e_ != cudaSuccess) {                                                     \
            set_error(std::string("kernel launch at batch.cu:") + std::to_string(__LINE__) + ": " + \
                      cudaGetErrorString(e_));                                       \
            return GBPF_E_CUDA;                                                      \
        }                                                                            \
    } while (0)

// ---------------------------------------------------------------------------
// learned warm start
// ---------------------------------------------------------------------------
// Network features of every instance, normalised, bf16: [Pliq | Qliq | V0]
// over the instance's buses, zero padding up to kin.
// Features [Pliq | Qliq | V0] of every instance (n_in = 3 nB), or [Pliq |
// Qliq] (n_in = 2 nB), normalised, in bf16 rows of kin (zero padded).
// One block row of instances (blockIdx.y) and columns across the threads of
// blockIdx.x, so no thread divides a flat index by the row length.
__global__ void k_ws_features(const double *Pliq, const double *Qliq, const double *V0, const long long *inst_off,
                              int n_inst, int nB, int n_in, int kin, const float *mean, const float *iscale,
                              __nv_bfloat16 *X) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kin) return;
    const float mc = c < n_in ? mean[c] : 0.f, sc = c < n_in ? iscale[c] : 0.f;
    for (int inst = blockIdx.y; inst < n_inst; inst += gridDim.y) {
        const long long off = inst_off[inst];
        float v = 0.f;
        if (c < n_in) {
            const double x = c < nB ? Pliq[off + c] : c < 2 * nB ? Qliq[off + c - nB] : V0[off + c - 2 * nB];
            v = (float)((x - (double)mc) * (double)sc);
        }
        X[(long long)inst * kin + c] = __float2bfloat16_rn(v);
    }
}

// One block per instance: the predicted start (|V| of the PQ buses and theta
// of the non-slack buses from the network; the PV set points and the slack
// angle from the instance's own start) is kept when its initial mismatch --
// max |g| of the first Newton iteration: P rows of the non-slack buses, Q rows
// of the PQ buses, as in k_nr_block / k_nr_warp at iteration 0 -- is below
// that of the instance's own (flat) start; otherwise the own start is used.
// The two mismatches only rank the starts, so they are computed in FP32
// (phasors by sincosf, one pass over the Ybus rows for both starts); the
// shared flat iteration's P, Q (FP64) stand in for the own start's
// injections when the instances start from the grid's own state.  Writes
// the predicted start (FP64) to sV/sTh, kind[inst] = 1 (predicted) or 0,
// and the instance's queue class (k_ws_order) to cls_out, counted in hist.
// ef holds the FP32 phasors (V cos th, V sin th) of both starts, per bus.
constexpr int kSelThreads = 256;
constexpr int kOrderClasses = 64;
__device__ __forceinline__ unsigned fabits(float x) { return __float_as_uint(x) & 0x7fffffffu; }
__device__ __forceinline__ unsigned warp_umax32(unsigned v) { return __reduce_max_sync(0xffffffffu, v); }
// SH: the phasors of the instance's two starts live in dynamic shared memory
// (16 B per bus) for the row gathers; otherwise in ef (global).
template <bool SH>
__global__ void __launch_bounds__(kSelThreads) k_ws_select(Args a, const float *pred, int ldp, const float *omean,
                                                           const float *oscale, double *sV, double *sTh, float4 *ef,
                                                           int *kind, int *cls_out, int *hist) {
    extern __shared__ float4 sel_ef[];
    __shared__ unsigned red[2][kSelThreads / 32];
    __shared__ float tred[2][kSelThreads / 32];
    const int inst = blockIdx.x, tid = threadIdx.x;
    const Topo T = a.topo[a.inst_topo[inst]];
    const TopoView G = bind(T.o, T.blob);
    const long long off = a.inst_off[inst];
    const int nB = T.nB;
    const float *pr = pred + (size_t)inst * ldp;
    float4 *e = SH ? sel_ef : ef + off;
    const char *flat = (T.flat && a.flat_on && *a.flat_on) ? T.flat : nullptr;
    const FlatLayout F = flat_layout<float>(nB, T.n + 2 * T.nup);  // P, Q offsets do not depend on the precision
    float tlo = INFINITY, thi = -INFINITY;  // spread of the predicted angles
    for (int k = tid; k < nB; k += kSelThreads) {
        const int ty = G.type[k];
        // the own start: the grid's (the shared flat copy, read by every
        // instance from L2) when the instances start from it
        const double v0 = flat ? ((const double *)(flat + F.V0))[k] : a.V0[off + k];
        const double t0 = flat ? ((const double *)(flat + F.th0))[k] : a.th0[off + k];
        const double v = (ty == 0 || ty == 1) ? (double)pr[k] * oscale[k] + omean[k] : v0;
        const double t = ty == 3 ? t0 : (double)pr[nB + k] * oscale[nB + k] + omean[nB + k];
        sV[off + k] = v;
        sTh[off + k] = t;
        // NaN stays NaN through the spread and lands in the top class
        tlo = (float)t < tlo || t != t ? (float)t : tlo;
        thi = (float)t > thi || t != t ? (float)t : thi;
        float s, c, s0 = 0.f, c0 = 0.f;
        sincosf((float)t, &s, &c);
        if (!flat) sincosf((float)t0, &s0, &c0);
        e[k] = make_float4((float)v * c, (float)v * s, (float)v0 * c0, (float)v0 * s0);
    }
    __syncthreads();
    unsigned mp = 0, mf = 0;
    for (int k = tid; k < nB; k += kSelThreads) {
        const int ty = G.type[k];
        if (ty == 3) continue;
        float ir = 0.f, ii = 0.f, jr = 0.f, ji = 0.f;
        for (int p = G.yptr[k]; p < G.yptr[k + 1]; p++) {
            const float2 yf = G.yval32[p];  // the FP64 values rounded to FP32
            const float yr = yf.x, yi = yf.y;
            const float4 u = e[G.ycol[p]];
            ir = fmaf(yr, u.x, fmaf(-yi, u.y, ir));
            ii = fmaf(yr, u.y, fmaf(yi, u.x, ii));
            if (!flat) {
                jr = fmaf(yr, u.z, fmaf(-yi, u.w, jr));
                ji = fmaf(yr, u.w, fmaf(yi, u.z, ji));
            }
        }
        const float4 u = e[k];
        const double pl = a.Pliq[off + k];
        const float pf = flat ? (float)(pl - ((const double *)(flat + F.P))[k]) : (float)pl - fmaf(u.z, jr, u.w * ji);
        unsigned tp = fabits((float)pl - fmaf(u.x, ir, u.y * ii)), tf = fabits(pf);
        if (ty == 0 || ty == 1) {
            const double ql = a.Qliq[off + k];
            const float qf = flat ? (float)(ql - ((const double *)(flat + F.Q))[k]) : (float)ql - fmaf(u.w, jr, -u.z * ji);
            tp = max(tp, fabits((float)ql - fmaf(u.y, ir, -u.x * ii)));
            tf = max(tf, fabits(qf));
        }
        mp = max(mp, tp);
        mf = max(mf, tf);
    }
    mp = warp_umax32(mp);
    mf = warp_umax32(mf);
    for (int o = 16; o > 0; o >>= 1) {
        const float l = __shfl_xor_sync(0xffffffffu, tlo, o), h = __shfl_xor_sync(0xffffffffu, thi, o);
        tlo = l < tlo || l != l ? l : tlo;
        thi = h > thi || h != h ? h : thi;
    }
    if ((tid & 31) == 0) {
        red[0][tid >> 5] = mp;
        red[1][tid >> 5] = mf;
        tred[0][tid >> 5] = tlo;
        tred[1][tid >> 5] = thi;
    }
    __syncthreads();
    if (tid == 0) {
        for (int w = 1; w < kSelThreads / 32; w++) {
            mp = max(mp, red[0][w]);
            mf = max(mf, red[1][w]);
            tlo = tred[0][w] < tlo || tred[0][w] != tred[0][w] ? tred[0][w] : tlo;
            thi = tred[1][w] > thi || tred[1][w] != tred[1][w] ? tred[1][w] : thi;
        }
        // NaN patterns order above every number: a NaN predicted mismatch loses
        const bool use = mp < mf;
        kind[inst] = use ? 1 : 0;
        // The queue position class: the spread of the predicted angles, the
        // network's estimate of how stressed the scenario is.  Scenarios
        // beyond the point where Newton converges have the largest spreads
        // (measured on the 1,888-bus c5 scenarios: every non-converging one
        // ranked in the top 4 %, where ranking by load or by start mismatch
        // placed them at random), and they take the longest -- a failed
        // predicted run and then no_max_iter iterations -- so they go first.
        // Eight classes per binade over [2^-6, 4) rad (clamped; NaN on top).
        const float spread = thi - tlo;
        const unsigned key = spread != spread ? 0x7fc00000u : fabits(spread);
        const int cls = max(0, min(kOrderClasses - 1, (int)(key >> 20) - (121 << 3)));
        cls_out[inst] = cls;
        atomicAdd(&hist[cls], 1);
    }
}

// The work queue of a warm-started launch, by falling class (k_ws_select:
// the predicted angle spread): the instances expected to take longest -- a
// failed predicted run, then the full run from their own start -- are
// claimed first, so that they do not form the launch's tail.  hist[c] counts class c; cursor[] starts zeroed.  The
// order inside a class is whichever the atomics give: every instance's result
// is independent of its queue position.
__global__ void k_ws_order(const int *cls, const int *hist, int *cursor, int n_inst, int *queue) {
    __shared__ int start[kOrderClasses];
    if (threadIdx.x == 0) {
        int s = 0;
        for (int c = kOrderClasses - 1; c >= 0; c--) { start[c] = s; s += hist[c]; }
    }
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_inst; i += gridDim.x * blockDim.x) {
        const int c = cls[i];
        queue[start[c] + atomicAdd(&cursor[c], 1)] = i;
    }
}

// A converged run from the prediction is rejected (and the instance solved
// again from its own start) when a PQ bus's |V| lies more than this from the
// predicted start: Newton from a poor start can land on another solution of
// the power-flow equations (a low-voltage one), which the flat start avoids.
// Angles are not compared: a smooth angle offset in the prediction is cheap
// for Newton to remove and does not signal another solution.
constexpr double kWarmMaxDV = 0.05;
// Iterations a predicted start gets before it counts as failed: a start good
// enough to be chosen converges in a handful, and a failing one would
// otherwise hold its block for no_max_iter iterations before the fallback.
constexpr int kWarmMaxIter = 10;

// Owning device allocation (movable, not copyable).
struct DevBuf {
    void *p = nullptr;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p) { o.p = nullptr; }
    DevBuf &operator=(DevBuf &&o) noexcept {
        if (this != &o) { reset(); p = o.p; o.p = nullptr; }
        return *this;
    }
    void reset() { if (p) cudaFree(p); p = nullptr; }
    ~DevBuf() { reset(); }
};

}  // namespace

// Scratch of gbpf_batch_solve_noalloc: file-scope device memory, so that the
// entry point itself allocates nothing.  8 MiB on every GPU that loads the
// library, held until the process exits.  Every call shares it.
constexpr size_t kNoAllocBytes = 8u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
constexpr int kMaxDevices = 64;
// The table of sincos_tab -- cos and sin of 2 pi i / 256 in long double,
// rounded to double -- copied to the current device's symbol.  Every batch
// creation copies it (4 KB, identical bytes each time), so a device whose
// context was reset gets it again.
gbpf_status trig_table_setup() {
    static const std::vector<double2> table = [] {
        std::vector<double2> t(kTrigTab);
        const long double two_pi = 6.283185307179586476925286766559005768L;
        for (int i = 0; i < kTrigTab; i++) {
            const long double a = two_pi * i / kTrigTab;
            t[i] = make_double2((double)cosl(a), (double)sinl(a));
        }
        return t;
    }();
    CK(cudaMemcpyToSymbol(g_trig_tab, table.data(), sizeof(double2) * kTrigTab));
    return GBPF_OK;
}
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch for `device`, which must be current.  In
// host code the symbol is only a host-side stand-in, so the address comes
// from cudaGetSymbolAddress, once per device.
gbpf_status noalloc_setup(int device, void **out) {
    if (device < 0 || device >= kMaxDevices) { set_error("device ordinal out of range"); return GBPF_E_ARG; }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error(std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
            return GBPF_E_CUDA;
        }
        g_noalloc_ptr[device] = p;
    }
    *out = g_noalloc_ptr[device];
    return GBPF_OK;
}
}  // namespace

// Inputs of every instance packed on the device: V0, theta0, Pliq = Pg - Pload,
// Qliq = Qg - Qload and Qload, each bus from the caller's array when it was
// given (raw[q], copied up as they are: Pload, Qload, Pg, Qg, V0, theta0) or
// from its grid's own values (dflt, six arrays of nB per topology at
// dflt_off[t]).  One warp per instance.
struct PackArgs {
    const double *raw[6];
    const double *dflt;
    const long long *dflt_off;
    const Topo *topo;
    const int *inst_topo;
    const long long *inst_off;
    int n_inst;
    double *V0, *th0, *Pliq, *Qliq, *Qload;
};
__global__ void k_pack_inputs(PackArgs a) {
    const int inst = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (inst >= a.n_inst) return;
    const int t = a.inst_topo[inst];
    const int nB = a.topo[t].nB;
    const long long o = a.inst_off[inst];
    const double *d = a.dflt + a.dflt_off[t];
    for (int k = lane; k < nB; k += 32) {
        double v[6];
        for (int q = 0; q < 6; q++) v[q] = a.raw[q] ? a.raw[q][o + k] : d[(size_t)q * nB + k];
        a.Pliq[o + k] = v[2] - v[0];
        a.Qliq[o + k] = v[3] - v[1];
        a.Qload[o + k] = v[1];
        a.V0[o + k] = v[4];
        a.th0[o + k] = v[5];
    }
}

// ---------------------------------------------------------------------------
// host object
// ---------------------------------------------------------------------------
// The block kernel of a state placement level (layout gs), as a function
// handle for attributes and occupancy queries.
template <typename TJ> const void *warp_kernel(int gs) {
    if (gs == 3) return (const void *)k_nr_warp<TJ, 3>;
    if (gs == 2) return (const void *)k_nr_warp<TJ, 2>;
    if (gs == 1) return (const void *)k_nr_warp<TJ, 1>;
    return (const void *)k_nr_warp<TJ, 0>;
}
template <typename TJ> const void *blk_kernel(int gs) {
    if (gs == 3) return (const void *)k_nr_block<TJ, 3>;
    if (gs == 2) return (const void *)k_nr_block<TJ, 2>;
    if (gs == 1) return (const void *)k_nr_block<TJ, 1>;
    return (const void *)k_nr_block<TJ, 0>;
}

struct gbpf_batch {
    int device = 0;
    int precision = 0;
    double tol = 1e-8;
    int max_iter = 100, lim = 0, ev_cap = 16;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // warm-started solves in flight on several batches: step_done marks the
    // end of this batch's last warm-started solve (its result copies
    // included); follow_ev (another batch's step_done, set by
    // gbpf_batch_follow) is waited for on the device before this batch's next
    // warm-started solve starts.  Chaining whole solves keeps two Newton
    // launches from sharing the L2; letting the next solve's network and
    // start choice run beside the previous Newton launch's tail was measured
    // slower (466-467 k against 478 k solves/s one after the other on the
    // 1,888-bus scenarios: they share the same L2)
    cudaEvent_t step_done = nullptr, follow_ev = nullptr;
    // learned warm start: events after the network and after the start
    // choice, and the last call's phase times (network, choice, Newton)
    cudaEvent_t wev[2] = {nullptr, nullptr};
    cudaEvent_t pev[2] = {nullptr, nullptr};  // gbpf_batch_time_warm_pipelined: start, end
    float warm_ms[3] = {0, 0, 0};
    std::vector<Grid> grids;
    std::vector<YPattern> ys;
    std::vector<Symbolic> syms;
    std::vector<Topo> topo_h;
    std::vector<DevBuf> topo_mem;  // one allocation per topology
    DevBuf topo_d;
    // instances
    int n_inst = 0;
    long long n_bus_total = 0;
    std::vector<int> inst_topo;
    std::vector<long long> inst_off;
    DevBuf inst_mem, out_mem, scratch, counter, queues, handoff, topo_resume;
    int resume_region = 0;  // shared-memory bytes for the staged blob of a resumed instance
    Args args{};    // block-per-instance launch
    Args wargs{};   // warp-per-instance launch
    size_t smem = 0, warp_smem = 0, resume_smem = 0;
    int grid_blocks = 0, warp_grid = 0, warp_warps = 0, n_block_q = 0, n_warp_q = 0, resume_grid = 0;
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    // events around each kernel of the captured graph (block, warp, hand-off)
    cudaEvent_t kev[6] = {};
    DevBuf topo_na;                   // topologies planned for gbpf_batch_solve_noalloc
    DevBuf raw_mem;                   // the caller's input arrays as copied up (six of Σ nB)
    DevBuf dflt_mem;                  // the grids' own bus values, six arrays of nB per topology
    std::vector<long long> dflt_off;  // per topology, in doubles
    DevBuf dflt_off_d;
    int flat_flag = 0;                // host copy of the device flag behind Args::flat_on
    DevBuf flat_mem;                  // k_flat_start outputs, one FlatLayout per topology
    // the warm start's reference iteration (Args::wref): k_flat_start at the
    // network's mean output, with the PV set points and the slack angle of the
    // grid; made again when the mean, the grid or the lane grouping changes
    DevBuf wref_mem;
    const char *wref = nullptr;
    std::vector<float> wref_key;
    std::vector<double> wref_h;  // the reference state uploaded: |V|, then theta
    gbpf_status make_wref(const gbpf::MlpShape &sh, int t0);
    // gbpf_batch_solve_noalloc, per topology: shared memory of one instance
    // (whole state in shared memory) and the bytes of its factor slice
    std::vector<size_t> na_smem, na_stride;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;

    ~gbpf_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (step_done) cudaEventDestroy(step_done);
        for (auto &e : wev) if (e) cudaEventDestroy(e);
        for (auto &e : pev) if (e) cudaEventDestroy(e);
        if (mwork) gbpf::mlp_work_free(mwork);
        if (h_kind) cudaFreeHost(h_kind);
        if (h_witers) cudaFreeHost(h_witers);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        for (auto &e : kev) if (e) cudaEventDestroy(e);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }
    gbpf_status add_topology(const Grid &g);
    gbpf_status set_instances(int n, const int *topo_of_inst, const double *Pload, const double *Qload,
                              const double *Pg, const double *Qg, const double *V0, const double *th0);
    std::vector<int> topo_warp;  // per topology: served by k_nr_warp (1) or k_nr_block (0)
    // Launch plan (gbpf_batch_set_plan, gbpf_batch_autotune): warp_mode 0 puts
    // every instance on k_nr_block; warp_warps 0 = as many warps per block as
    // fit (8 by default: more warps per SM measured no faster on the 118-bus
    // batch); handoff_it 0 = no hand-off; resume_group / warp_group switch the
    // grouped lanes of deep levels in the hand-off blocks and in the warps;
    // narrow = 1 runs the narrow levels of the block kernel on one warp; lu1 /
    // warp_lu1 = 1 factor in one pass per elimination level in the block
    // kernel (block mode and hand-off) / in the warp kernel; flat_shared = 1
    // lets the warp kernel's instances take the shared iteration 0 of their
    // topology when they start from the grid's own state (k_flat_start);
    // rotate = 1 updates the FP32-LU form's phasors by rotation instead of a
    // sincos per iteration (measured slower on GB300, kept as a knob);
    // gstate = 1 lets the block kernel keep part of its state in global
    // memory (layout gs = 1 or 2, the latter also compiled for four blocks
    // per SM: level 3) where that fits more instances per SM or moves factors
    // into shared memory; 2, 3, 4 take level 1, 2, 3 wherever it fits; 0
    // never.
    struct Plan {
        int warp_mode = 1, warp_warps = 8, handoff_it = kHandoffIt, resume_group = 1, warp_group = 1, narrow = 0,
            lu1 = 1, warp_lu1 = 0, flat_shared = 1, rotate = 0, gstate = 1, warp_gstate = 1, quad = 1;
    } plan;
    int block_gs = 0;  // placement level of the block-mode launch's state (layout gs)
    int warp_gs = 0;   // ... and of the warp launch's
    DevBuf gstate_mem, warp_gstate_mem;
    gbpf_status rebuild() {
        CK(cudaStreamSynchronize(stream));
        if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
        if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
        return build_graph();
    }
    gbpf_status autotune(int repeats, float *best_ms, float *first_ms);
    // state and factor of one instance fit a warp's slice of shared memory
    bool warp_fits(const Topo &T) const {
        const bool fp32 = precision == GBPF_PREC_FP32_IR;
        const Layout w = fp32 ? layout<float>(T.nB, T.n, T.nup, T.nPV, 1, plan.warp_lu1)
                              : layout<double>(T.nB, T.n, T.nup, T.nPV, 1, plan.warp_lu1);
        return w.total <= (fp32 ? 40u : 56u) * 1024;
    }
    // learned warm start (solve_warm): features, prediction, chosen start, queue order
    DevBuf warm_mem;
    int warm_n = 0;
    __nv_bfloat16 *wX = nullptr;
    float *wPred = nullptr;
    double *wV = nullptr, *wTh = nullptr;
    float4 *wEF = nullptr;
    int *wKind = nullptr, *wQueue = nullptr, *wIters = nullptr, *wCls = nullptr, *wHist = nullptr;
    gbpf_status launch(cudaStream_t st);
    gbpf_status launch_with(cudaStream_t st, const Args &ba, const Args &wa, bool timed = false);
    gbpf_status build_graph();
    gbpf_status solve_warm(gbpf_mlp *m, int *kind, int *warm_iters, float *ms);
    // the same in two halves: everything enqueued on the batch stream, then
    // the wait and the per-instance start kinds
    gbpf_status warm_launch(gbpf_mlp *m);
    gbpf_status warm_wait(int *kind, int *warm_iters, float *ms);
    gbpf::MlpWork *mwork = nullptr;      // the network's activations for this batch
    int *h_kind = nullptr, *h_witers = nullptr;  // pinned copies of wKind, wIters
    bool warm_pending = false;
};

gbpf_status gbpf_batch::add_topology(const Grid &g) {
    if (g.nB < 2 || g.slack < 1) { set_error("grid needs at least two buses and one slack"); return GBPF_E_INPUT; }
    for (int b = 0; b < g.nL; b++)
        if (g.r[b] == 0.0 && g.x[b] == 0.0) { set_error("branch with zero impedance"); return GBPF_E_INPUT; }
    YPattern y = gbpf::build_ypattern(g);
    std::string why;
    Symbolic S = gbpf::analyse(g, y, &why);
    if (S.n != g.nB - 1) { set_error("symbolic analysis failed: " + why); return GBPF_E_INPUT; }
    if (S.pairs() >= (1LL << 31)) { set_error("factor too large for the batched kernel"); return GBPF_E_UNSUPPORTED; }
    const int nB = g.nB, nL = g.nL, n = S.n, nup = S.nup, nq = n + 2 * nup, nfl = (int)S.flev_ptr.size() - 1,
              nbl = (int)S.blev_ptr.size() - 1;
    std::vector<int> pv0(g.nPV), ogp(nup + 1);
    for (int i = 0; i < g.nPV; i++) pv0[i] = g.pv[i] - 1;
    for (int p = 0; p <= nup; p++) ogp[p] = (int)S.og_ptr[p];
    // the blob: every read-only array of the topology, 16-byte aligned pieces
    std::vector<char> blob;
    auto put = [&](const void *src, size_t bytes) {
        const size_t o = align_up(blob.size(), 16);
        blob.resize(align_up(o + bytes, 16), 0);
        if (src && bytes) std::memcpy(blob.data() + o, src, bytes);
        return (int)o;
    };
    TopoOff o;
    o.yptr = put(y.rowptr.data(), (nB + 1) * 4); o.ycol = put(y.col.data(), y.nnz * 4);
    o.yval = put(nullptr, (size_t)y.nnz * 16);
    o.type = put(g.type.data(), nB * 4); o.pv_bus = put(pv0.data(), g.nPV * 4);
    o.Qmin = put(g.Qmin.data(), g.nPV * 8); o.Qmax = put(g.Qmax.data(), g.nPV * 8);
    o.bus_of_blk = put(S.bus_of_blk.data(), n * 4); o.up_ptr = put(S.up_ptr.data(), (n + 1) * 4);
    o.up_col = put(S.up_col.data(), nup * 4); o.dg_ptr = put(S.dg_ptr.data(), (n + 1) * 4);
    o.dg_pos = put(S.dg_pos.data(), nup * 4); o.dg_k = put(S.dg_k.data(), nup * 4);
    o.og_ptr = put(ogp.data(), (nup + 1) * 4);
    o.og_a = put(S.og_a.data(), S.og_a.size() * 4); o.og_b = put(S.og_b.data(), S.og_b.size() * 4);
    o.flev_ptr = put(S.flev_ptr.data(), (nfl + 1) * 4); o.flev_steps = put(S.flev_steps.data(), n * 4);
    o.blev_ptr = put(S.blev_ptr.data(), (nbl + 1) * 4); o.blev_steps = put(S.blev_steps.data(), n * 4);
    o.ysl = put(S.ysl.data(), nq * 4); o.rbus = put(S.rbus.data(), nq * 4); o.cbus = put(S.cbus.data(), nq * 4);
    o.fent_ptr = put(S.fent_ptr.data(), (nfl + 1) * 4); o.fent_p = put(S.fent_p.data(), nup * 4);
    o.fent_j = put(S.fent_j.data(), nup * 4);
    // lanes per pivot / entry / row of each level for the block kernel: as many
    // as the level's thread budget allows, no more than its longest list needs
    // (grp), and the same for the 32 lanes of the warp kernel (grpw)
    std::vector<int> grp(3 * (size_t)std::max(nfl, nbl), 0), grpw(grp.size(), 0);
    auto group_of = [](int count, int longest, int threads) {
        int g = 0;
        while (g < 5 && ((long long)count << (g + 1)) <= threads && (1 << g) < longest) g++;
        return g;
    };
    for (int l = 0; l < nfl; l++) {
        int md = 0, mo = 0;
        for (int w = S.flev_ptr[l]; w < S.flev_ptr[l + 1]; w++) {
            const int j = S.flev_steps[w];
            md = std::max(md, S.dg_ptr[j + 1] - S.dg_ptr[j]);
        }
        for (int e = S.fent_ptr[l]; e < S.fent_ptr[l + 1]; e++) {
            const int pp = S.fent_p[e];
            mo = std::max(mo, (int)(S.og_ptr[pp + 1] - S.og_ptr[pp]));
        }
        for (int w = 0; w < 2; w++) {
            std::vector<int> &gv = w ? grpw : grp;
            const int th = w ? 32 : kThreads;
            gv[3 * l] = group_of(S.flev_ptr[l + 1] - S.flev_ptr[l], md, th);
            gv[3 * l + 1] = group_of(S.fent_ptr[l + 1] - S.fent_ptr[l], mo, th);
        }
    }
    for (int l = 0; l < nbl; l++) {
        int mu = 0;
        for (int w = S.blev_ptr[l]; w < S.blev_ptr[l + 1]; w++) {
            const int j = S.blev_steps[w];
            mu = std::max(mu, S.up_ptr[j + 1] - S.up_ptr[j]);
        }
        grp[3 * l + 2] = group_of(S.blev_ptr[l + 1] - S.blev_ptr[l], mu, kThreads);
        grpw[3 * l + 2] = group_of(S.blev_ptr[l + 1] - S.blev_ptr[l], mu, 32);
    }
    o.lvl_group = put(grp.data(), grp.size() * 4);
    o.lvl_group_w = put(grpw.data(), grpw.size() * 4);
    std::vector<int> narrow(std::max(nfl, nbl), 0);
    for (int l = 0; l < nfl; l++)
        if (S.flev_ptr[l + 1] - S.flev_ptr[l] <= 32 && S.fent_ptr[l + 1] - S.fent_ptr[l] <= 32) narrow[l] |= 1;
    for (int l = 0; l < nbl; l++)
        if (S.blev_ptr[l + 1] - S.blev_ptr[l] <= 32) narrow[l] |= 2;
    o.lvl_narrow = put(narrow.data(), narrow.size() * 4);
    // one-pass levels: the entries start past the lanes the pivots occupy
    std::vector<int> rot(std::max(nfl, 1), 0);
    for (int l = 0; l < nfl; l++) {
        const int np = S.flev_ptr[l + 1] - S.flev_ptr[l];
        const long long pb = (long long)np << grp[3 * l], pw = (long long)np << grpw[3 * l];
        const int rb = pb < kThreads ? (int)align_up((size_t)pb, 32) : 0;
        const int rw = (pw <= 16 && grpw[3 * l + 1] <= 4) ? 16 : 0;
        rot[l] = (rb % kThreads) | (rw << 16);
    }
    o.lvl_rot = put(rot.data(), rot.size() * 4);
    o.og_k = put(S.og_k.data(), S.og_k.size() * 4);
    o.yval32 = put(nullptr, (size_t)y.nnz * 8);
    // lu_level1_q: quads per pivot / entry (at most eight, a warp) for the
    // block kernel's kThreads / 4 quads, and the entries' rotation past the
    // pivots' threads
    std::vector<int> grp4(2 * (size_t)std::max(nfl, 1), 0), rot4(std::max(nfl, 1), 0);
    std::vector<int> grp4w(grp4.size(), 0), q4w(rot4.size(), 0);
    for (int l = 0; l < nfl; l++) {
        int md = 0, mo = 0;
        for (int w = S.flev_ptr[l]; w < S.flev_ptr[l + 1]; w++) {
            const int j = S.flev_steps[w];
            md = std::max(md, S.dg_ptr[j + 1] - S.dg_ptr[j]);
        }
        for (int e = S.fent_ptr[l]; e < S.fent_ptr[l + 1]; e++) {
            const int pp = S.fent_p[e];
            mo = std::max(mo, (int)(S.og_ptr[pp + 1] - S.og_ptr[pp]));
        }
        auto g4 = [](int count, int longest, int quads = kThreads / 4) {
            int g = 0;
            while (g < 3 && ((long long)count << (g + 1)) <= quads && (1 << g) < longest) g++;
            return g;
        };
        const int np = S.flev_ptr[l + 1] - S.flev_ptr[l], ne = S.fent_ptr[l + 1] - S.fent_ptr[l];
        grp4[2 * l] = g4(np, md);
        grp4[2 * l + 1] = g4(ne, mo);
        const long long pt = ((long long)np << grp4[2 * l]) * 4;  // threads the pivots occupy
        rot4[l] = pt < kThreads ? (int)(align_up((size_t)pt, 32) % kThreads) : 0;
        // quads only where the level's pivots and entries each fit one pass of
        // the block's quads and no quad walks more than 16 elements of a gather
        // list: a wider level already fills the lanes one thread a block, and
        // a longer walk is a longer dependent chain (rot4 = -1: one lane a
        // block).  Measured FP64 solves: quads wherever a level fits took the
        // 118-bus grids 0.35 -> 0.27 ms and 1,888 buses 1.63 -> 1.52 ms, but a
        // 472-bus grid whose deep levels walk 26-57 elements a quad 9.5 -> 10.8
        auto walk = [](int longest, int g) { return (longest + (1 << g) - 1) >> g; };
        if (((long long)np << grp4[2 * l]) > kThreads / 4 || ((long long)ne << grp4[2 * l + 1]) > kThreads / 4 ||
            walk(md, grp4[2 * l]) > 16 || walk(mo, grp4[2 * l + 1]) > 16)
            rot4[l] = -1;
        // the warp's eight quads, by the same rule
        grp4w[2 * l] = g4(np, md, 8);
        grp4w[2 * l + 1] = g4(ne, mo, 8);
        q4w[l] = ((long long)np << grp4w[2 * l]) <= 8 && ((long long)ne << grp4w[2 * l + 1]) <= 8 &&
                 walk(md, grp4w[2 * l]) <= 16 && walk(mo, grp4w[2 * l + 1]) <= 16;
    }
    o.lvl_group4 = put(grp4.data(), grp4.size() * 4);
    // injection row order: a warp's loop runs to its longest row, so rows of
    // the same length go together (measured on the 1,888-bus grid: 1.84x the
    // needed row steps in bus order)
    std::vector<int> order(nB);
    for (int k = 0; k < nB; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        return y.rowptr[a + 1] - y.rowptr[a] > y.rowptr[c + 1] - y.rowptr[c];
    });
    o.inj_order = put(order.data(), nB * 4);
    o.lvl_rot4 = put(rot4.data(), rot4.size() * 4);
    o.lvl_group4w = put(grp4w.data(), grp4w.size() * 4);
    o.lvl_q4w = put(q4w.data(), q4w.size() * 4);
    DevBuf mem, tmp;
    CK(cudaMalloc(&mem.p, blob.size()));
    CK(cudaMemcpyAsync(mem.p, blob.data(), blob.size(), cudaMemcpyHostToDevice, stream));
    // Ybus values into the blob, assembled on the device (calcYbusSp_eficinte or
    // calcYbusSp_Matpower, by the grid's form)
    size_t used = 0;
    auto tk = [&](size_t bytes) { used = align_up(used, 256); size_t r = used; used += bytes; return r; };
    const size_t t_cptr = tk((y.nnz + 1) * 4), t_csrc = tk(y.csrc.size() * 4), t_stamp = tk(16 * (size_t)(4 * nL + 1));
    const size_t t_r = tk(nL * 8 + 8), t_x = tk(nL * 8 + 8), t_b = tk(nL * 8 + 8), t_tre = tk(nL * 8 + 8),
                 t_tim = tk(nL * 8 + 8), t_gsh = tk(nB * 8), t_bsh = tk(nB * 8);
    CK(cudaMalloc(&tmp.p, used + 256));
    char *tb = (char *)tmp.p;
    CK(cudaMemcpyAsync(tb + t_cptr, y.cptr.data(), (y.nnz + 1) * 4, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(tb + t_csrc, y.csrc.data(), y.csrc.size() * 4, cudaMemcpyHostToDevice, stream));
    if (nL) {
        CK(cudaMemcpyAsync(tb + t_r, g.r.data(), nL * 8, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(tb + t_x, g.x.data(), nL * 8, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(tb + t_b, g.bch.data(), nL * 8, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(tb + t_tre, g.tap_re.data(), nL * 8, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(tb + t_tim, g.tap_im.data(), nL * 8, cudaMemcpyHostToDevice, stream));
    }
    CK(cudaMemcpyAsync(tb + t_gsh, g.gsh.data(), nB * 8, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(tb + t_bsh, g.bsh.data(), nB * 8, cudaMemcpyHostToDevice, stream));
    if (nL) k_batch_stamps<<<(nL + 255) / 256, 256, 0, stream>>>((const double *)(tb + t_r), (const double *)(tb + t_x),
                                                                 (const double *)(tb + t_b), (const double *)(tb + t_tre),
                                                                 (const double *)(tb + t_tim), (double2 *)(tb + t_stamp), nL,
                                                                 g.ybus_form);
    k_batch_ybus<<<(y.nnz + 255) / 256, 256, 0, stream>>>((const int *)(tb + t_cptr), (const int *)(tb + t_csrc),
                                                          (const double2 *)(tb + t_stamp), (const double *)(tb + t_gsh),
                                                          (const double *)(tb + t_bsh),
                                                          (double2 *)((char *)mem.p + o.yval),
                                                          (float2 *)((char *)mem.p + o.yval32), y.nnz);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(stream));
    Topo t{};
    t.nB = nB; t.nL = nL; t.n = n; t.nup = nup; t.nnzY = y.nnz; t.nPV = g.nPV; t.nfl = nfl; t.nbl = nbl;
    t.blob_bytes = (int)blob.size();
    t.blob = (const char *)mem.p;
    t.o = o;
    grids.push_back(g);
    ys.push_back(std::move(y));
    syms.push_back(std::move(S));
    topo_h.push_back(t);
    topo_mem.push_back(std::move(mem));
    return GBPF_OK;
}

gbpf_status gbpf_batch::set_instances(int n, const int *tofi, const double *Pload, const double *Qload,
                                      const double *Pg, const double *Qg, const double *V0, const double *th0) {
    if (warm_pending) { set_error("a warm-started solve is in flight: wait for it first"); return GBPF_E_ARG; }
    for (int i = 0; i < n; i++)
        if (tofi[i] < 0 || tofi[i] >= (int)grids.size()) { set_error("instance names an unknown grid"); return GBPF_E_ARG; }
    const bool same = exec && n == n_inst && std::equal(tofi, tofi + n, inst_topo.begin());
    if (!same) {
        CK(cudaStreamSynchronize(stream));
        n_inst = n;
        inst_topo.assign(tofi, tofi + n);
        inst_off.resize(n);
        long long off = 0;
        for (int i = 0; i < n; i++) {
            inst_off[i] = off;
            off += grids[inst_topo[i]].nB;
        }
        n_bus_total = off;
    }
    const size_t nb = (size_t)n_bus_total * 8, nba = align_up(nb, 256);
    if (!same) {
        // inputs: V0, th0, Pliq, Qliq, Qload (packed, one device region) and
        // the caller's raw arrays; outputs: V, th, P, Q + per-instance results
        inst_mem.reset();
        out_mem.reset();
        raw_mem.reset();
        const size_t in_bytes = 5 * nba + align_up(4 * (size_t)n, 256) + align_up(8 * (size_t)n, 256);
        CK(cudaMalloc(&inst_mem.p, in_bytes));
        CK(cudaMalloc(&raw_mem.p, 6 * nba));
        char *bb = (char *)inst_mem.p;
        size_t o = 0;
        auto take = [&](size_t bytes) { char *r = bb + o; o += align_up(bytes, 256); return r; };
        args.V0 = (double *)take(nb); args.th0 = (double *)take(nb); args.Pliq = (double *)take(nb);
        args.Qliq = (double *)take(nb); args.Qload = (double *)take(nb);
        args.inst_topo = (int *)take(4 * (size_t)n);
        args.inst_off = (long long *)take(8 * (size_t)n);
        CK(cudaMemcpyAsync((void *)args.inst_topo, inst_topo.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync((void *)args.inst_off, inst_off.data(), 8 * (size_t)n, cudaMemcpyHostToDevice, stream));
        const size_t out_bytes = 4 * nba + 3 * align_up(4 * (size_t)n, 256) + align_up(8 * (size_t)n, 256);
        const size_t ev_bytes = align_up(16 * (size_t)n * ev_cap, 256);
        CK(cudaMalloc(&out_mem.p, out_bytes + ev_bytes));
        bb = (char *)out_mem.p;
        o = 0;
        args.V = (double *)take(nb); args.th = (double *)take(nb); args.P = (double *)take(nb); args.Q = (double *)take(nb);
        args.iters = (int *)take(4 * (size_t)n); args.status = (int *)take(4 * (size_t)n);
        args.n_events = (int *)take(4 * (size_t)n); args.mism = (double *)take(8 * (size_t)n);
        args.events = (int *)take(16 * (size_t)n * ev_cap);
        args.n_inst = n;
        CK(cudaStreamSynchronize(stream));
        if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
        if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
        const gbpf_status st = build_graph();
        if (st != GBPF_OK) return st;
    }
    // the caller's arrays go up as they are (one copy each; on a GPU that
    // reads pageable host memory through the host page tables, as GB300 does,
    // at the rate of a pinned copy); the packing runs on the device
    const double *user[6] = {Pload, Qload, Pg, Qg, V0, th0};
    PackArgs pa{};
    for (int q = 0; q < 6; q++) {
        if (!user[q]) continue;
        double *dst = (double *)((char *)raw_mem.p + q * nba);
        CK(cudaMemcpyAsync(dst, user[q], nb, cudaMemcpyHostToDevice, stream));
        pa.raw[q] = dst;
    }
    pa.dflt = (const double *)dflt_mem.p;
    pa.dflt_off = (const long long *)dflt_off_d.p;
    pa.topo = (const Topo *)topo_d.p;
    pa.inst_topo = args.inst_topo;
    pa.inst_off = args.inst_off;
    pa.n_inst = n;
    pa.V0 = (double *)args.V0; pa.th0 = (double *)args.th0; pa.Pliq = (double *)args.Pliq;
    pa.Qliq = (double *)args.Qliq; pa.Qload = (double *)args.Qload;
    k_pack_inputs<<<(unsigned)(((long long)n * 32 + 255) / 256), 256, 0, stream>>>(pa);
    CK_LAUNCH();
    // instances from the grids' own start may take the shared iteration 0
    flat_flag = (!V0 && !th0) ? 1 : 0;
    CK(cudaMemcpyAsync((int *)counter.p + 8, &flat_flag, sizeof(int), cudaMemcpyHostToDevice, stream));
    // the caller may reuse its arrays on return, pinned ones included
    CK(cudaStreamSynchronize(stream));
    return GBPF_OK;
}

gbpf_status gbpf_batch::launch(cudaStream_t st) { return launch_with(st, args, wargs, true); }

// One persistent launch per mode over the queues of ba (blocks) and wa (warps).
gbpf_status gbpf_batch::launch_with(cudaStream_t st, const Args &ba, const Args &wa, bool timed) {
    const bool fp32 = precision == GBPF_PREC_FP32_IR;
    CK(cudaMemsetAsync(args.counter, 0, 4 * sizeof(int), st));
    if (ba.queue_len) {
        CK(cudaEventRecord(fork, st));
        CK(cudaStreamWaitEvent(side, fork, 0));
        if (timed) CK(cudaEventRecordWithFlags(kev[0], side, cudaEventRecordExternal));
        if (fp32) {
            if (block_gs == 3) k_nr_block<float, 3><<<grid_blocks, kThreads, smem, side>>>(ba);
            else if (block_gs == 2) k_nr_block<float, 2><<<grid_blocks, kThreads, smem, side>>>(ba);
            else if (block_gs == 1) k_nr_block<float, 1><<<grid_blocks, kThreads, smem, side>>>(ba);
            else k_nr_block<float, 0><<<grid_blocks, kThreads, smem, side>>>(ba);
        } else {
            if (block_gs == 3) k_nr_block<double, 3><<<grid_blocks, kThreads, smem, side>>>(ba);
            else if (block_gs == 2) k_nr_block<double, 2><<<grid_blocks, kThreads, smem, side>>>(ba);
            else if (block_gs == 1) k_nr_block<double, 1><<<grid_blocks, kThreads, smem, side>>>(ba);
            else k_nr_block<double, 0><<<grid_blocks, kThreads, smem, side>>>(ba);
        }
        {
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                cudaFuncAttributes fa{};
                cudaFuncGetAttributes(&fa, fp32 ? blk_kernel<float>(block_gs) : blk_kernel<double>(block_gs));
                set_error(std::string("k_nr_block launch (") + std::to_string(grid_blocks) + " blocks, " +
                          std::to_string(smem) + " B dynamic shared memory; the kernel allows " +
                          std::to_string(fa.maxDynamicSharedSizeBytes) + " B dynamic, " +
                          std::to_string(fa.sharedSizeBytes) + " B static, " + std::to_string(fa.numRegs) +
                          " registers, " + std::to_string(fa.localSizeBytes) + " B local): " + cudaGetErrorString(e));
                return GBPF_E_CUDA;
            }
        }
        if (timed) CK(cudaEventRecordWithFlags(kev[1], side, cudaEventRecordExternal));
    }
    if (wa.queue_len) {
        if (timed) CK(cudaEventRecordWithFlags(kev[2], st, cudaEventRecordExternal));
        const dim3 wg(warp_grid), wb(32 * warp_warps);
        if (fp32) {
            if (warp_gs == 3) k_nr_warp<float, 3><<<wg, wb, warp_smem, st>>>(wa);
            else if (warp_gs == 2) k_nr_warp<float, 2><<<wg, wb, warp_smem, st>>>(wa);
            else if (warp_gs == 1) k_nr_warp<float, 1><<<wg, wb, warp_smem, st>>>(wa);
            else k_nr_warp<float, 0><<<wg, wb, warp_smem, st>>>(wa);
        } else {
            if (warp_gs == 3) k_nr_warp<double, 3><<<wg, wb, warp_smem, st>>>(wa);
            else if (warp_gs == 2) k_nr_warp<double, 2><<<wg, wb, warp_smem, st>>>(wa);
            else if (warp_gs == 1) k_nr_warp<double, 1><<<wg, wb, warp_smem, st>>>(wa);
            else k_nr_warp<double, 0><<<wg, wb, warp_smem, st>>>(wa);
        }
        CK_LAUNCH();
        if (timed) CK(cudaEventRecordWithFlags(kev[3], st, cudaEventRecordExternal));
        if (wa.handoff_it > 0) {
            // the instances the warps parked, one block each, same arithmetic
            Args ra = wa;
            ra.resume = 1;
            ra.no_group = plan.resume_group ? 0 : 1;
            ra.narrow = plan.narrow;
            ra.lu1 = plan.lu1;
            ra.quad = plan.quad;
            ra.rotate = plan.rotate;
            ra.queue = wa.handoff_q;
            ra.counter = args.counter + 2;
            ra.topo = (const Topo *)topo_resume.p;
            ra.blob_region = resume_region;
            if (fp32) k_nr_block<float, 0><<<resume_grid, kThreads, resume_smem, st>>>(ra);
            else k_nr_block<double, 0><<<resume_grid, kThreads, resume_smem, st>>>(ra);
            CK_LAUNCH();
            if (timed) CK(cudaEventRecordWithFlags(kev[4], st, cudaEventRecordExternal));
        }
    }
    if (ba.queue_len) {
        CK(cudaEventRecord(join, side));
        CK(cudaStreamWaitEvent(st, join, 0));
    }
    return GBPF_OK;
}

gbpf_status gbpf_batch::build_graph() {
    const bool fp32 = precision == GBPF_PREC_FP32_IR;
    int dev_sm = 0, maxsm = 0;
    CK(cudaDeviceGetAttribute(&dev_sm, cudaDevAttrMultiProcessorCount, device));
    CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    // Warp-per-instance for topologies whose state and factor fit a warp slice
    // of shared memory; block-per-instance (factor possibly in scratch) else.
    std::vector<int> warp_ok(topo_h.size(), 0);
    size_t slice = 0;
    for (size_t t = 0; t < topo_h.size(); t++) {
        const Topo &T = topo_h[t];
        if (plan.warp_mode && warp_fits(T)) {
            warp_ok[t] = 1;
            const Layout w = fp32 ? layout<float>(T.nB, T.n, T.nup, T.nPV, 1, plan.warp_lu1)
                                  : layout<double>(T.nB, T.n, T.nup, T.nPV, 1, plan.warp_lu1);
            slice = std::max(slice, align_up(w.total, 128));
        }
    }
    topo_warp = warp_ok;
    std::vector<int> wq, bq;
    for (int i = 0; i < n_inst; i++) (warp_ok[inst_topo[i]] ? wq : bq).push_back(i);
    n_warp_q = (int)wq.size();
    n_block_q = (int)bq.size();
    queues.reset();
    CK(cudaMalloc(&queues.p, 4 * (size_t)n_inst + 256));
    if (n_warp_q) CK(cudaMemcpy(queues.p, wq.data(), 4 * wq.size(), cudaMemcpyHostToDevice));
    if (n_block_q) CK(cudaMemcpy((int *)queues.p + n_warp_q, bq.data(), 4 * bq.size(), cudaMemcpyHostToDevice));
    // Block-mode shared-memory plan: the blob is staged in shared memory when
    // at most 48 KB; the factor stays in shared memory when blob region +
    // state + factor fit in 110 KB, otherwise it lives in global scratch.
    // With plan.gstate the plan is also made with part of the state in global
    // memory (layout gs), and that one is taken when it fits more blocks per
    // SM, or as many with more factors in shared memory.
    const size_t budget = 110 * 1024, blob_cap = 48 * 1024;
    size_t region = 0;
    for (size_t t = 0; t < topo_h.size(); t++) {
        Topo &T = topo_h[t];
        T.blob_smem = !warp_ok[t] && (size_t)T.blob_bytes <= blob_cap;
        if (T.blob_smem) region = std::max(region, align_up((size_t)T.blob_bytes, 32));
    }
    auto blk_fn = [&](int gs) -> const void * {
        if (fp32) return blk_kernel<float>(gs);
        return blk_kernel<double>(gs);
    };
    struct BlockPlan {
        size_t need = 0, scr = 0, gst = 0;
        std::vector<int> fac;
        int nfac = 0, occ = 0;
    };
    auto plan_blocks = [&](int gs, size_t budget, BlockPlan &bp) -> gbpf_status {
        bp.fac.assign(topo_h.size(), 1);
        for (size_t t = 0; t < topo_h.size(); t++) {
            if (warp_ok[t]) continue;
            const Topo &T = topo_h[t];
            const int z = plan.lu1;
            const int lv = std::min(gs, 2);
            const Layout with = fp32 ? layout<float>(T.nB, T.n, T.nup, T.nPV, 1, z, lv)
                                     : layout<double>(T.nB, T.n, T.nup, T.nPV, 1, z, lv);
            const Layout without = fp32 ? layout<float>(T.nB, T.n, T.nup, T.nPV, 0, z, lv)
                                        : layout<double>(T.nB, T.n, T.nup, T.nPV, 0, z, lv);
            bp.gst = std::max(bp.gst, with.gtotal);
            if (region + with.total <= budget) {
                bp.nfac++;
                bp.need = std::max(bp.need, with.total);
            } else {
                bp.fac[t] = 0;
                bp.need = std::max(bp.need, without.total);
                bp.scr = std::max(bp.scr, fp32 ? scratch_bytes<float>(T.n, T.nup) : scratch_bytes<double>(T.n, T.nup));
            }
        }
        const size_t sm = bp.need + region;
        if (!n_block_q || sm > (size_t)maxsm) return GBPF_OK;
        CK(cudaFuncSetAttribute(blk_fn(gs), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bp.occ, blk_fn(gs), kThreads, sm));
        return GBPF_OK;
    };
    // Placement level: gstate 2 / 3 / 4 take level 1 / 2 / 3 where it fits;
    // gstate 1 a level with at least 1.5x the blocks per SM (global state
    // costs latency, which only more blocks per SM win back), else one with
    // as many and more factors in shared memory, else the lower.  Measured on
    // 8,192 instances of a 1,888-bus grid (solves/s): FP32 level 0 124 k
    // (1 block per SM), 1 194 k (2), 2 199 k (2), 3 290 k (4; 259 k at 3,
    // 279 k at 5 and 217 k at 6 blocks per SM, where spills grow), and 133 k with the factor
    // given the whole of shared memory at 1 block per SM; FP64 57 k, 58 k,
    // 71 k, 71 k (3 blocks per SM).
    BlockPlan bp;
    gbpf_status pst = plan_blocks(0, budget, bp);
    if (pst != GBPF_OK) return pst;
    block_gs = 0;
    if (plan.gstate && n_block_q) {
        for (int gs = 1; gs <= 3; gs++) {
            BlockPlan c;
            if ((pst = plan_blocks(gs, budget, c)) != GBPF_OK) return pst;
            const bool take = plan.gstate >= 2 ? (gs == plan.gstate - 1 && c.occ > 0)
                                               : (2 * c.occ >= 3 * bp.occ && c.occ > 0) ||
                                                     (c.occ == bp.occ && c.occ > 0 && c.nfac > bp.nfac);
            if (take) {
                bp = c;
                block_gs = gs;
            }
        }
    }
    for (size_t t = 0; t < topo_h.size(); t++) topo_h[t].fac_smem = bp.fac[t];
    const size_t need = bp.need, scr = bp.scr;
    args.blob_region = (int)region;
    smem = n_block_q ? need + region : 0;
    if (smem > (size_t)maxsm) { set_error("instance state does not fit in shared memory"); return GBPF_E_UNSUPPORTED; }
    // stragglers of the warp kernel resume on blocks with their factor and,
    // when it fits next to the state, the topology's blob in shared memory
    // (few instances per SM get that far, so shared memory is not scarce)
    resume_smem = 0;
    resume_region = 0;
    std::vector<Topo> rt(topo_h);
    {
        size_t state = 0, region_r = 0;
        for (size_t t = 0; t < topo_h.size(); t++) {
            if (!warp_ok[t]) continue;
            const Topo &T = topo_h[t];
            state = std::max(state, fp32 ? layout<float>(T.nB, T.n, T.nup, T.nPV, 1, plan.lu1).total
                                         : layout<double>(T.nB, T.n, T.nup, T.nPV, 1, plan.lu1).total);
            region_r = std::max(region_r, align_up((size_t)T.blob_bytes, 32));
        }
        const bool stage = state + region_r <= (size_t)maxsm;
        for (size_t t = 0; t < rt.size(); t++) {
            rt[t].fac_smem = 1;
            rt[t].blob_smem = warp_ok[t] && stage;
        }
        resume_region = stage ? (int)region_r : 0;
        resume_smem = state + resume_region;
    }
    const bool use_handoff = n_warp_q > 0 && plan.handoff_it > 0 && max_iter > plan.handoff_it;
    grid_blocks = 0;
    resume_grid = 0;
    {
        // the resume launch always keeps its state in shared memory
        size_t attr_sm = use_handoff ? resume_smem : 0;
        if (!block_gs) attr_sm = std::max(attr_sm, smem);
        if (attr_sm) CK(cudaFuncSetAttribute(blk_fn(0), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)attr_sm));
        if (block_gs) CK(cudaFuncSetAttribute(blk_fn(block_gs), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    if (n_block_q) {
        int occ = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, blk_fn(block_gs), kThreads, smem));
        grid_blocks = std::max(1, std::min(n_block_q, dev_sm * std::max(occ, 1)));
    }
    if (use_handoff) {
        int occ = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, blk_fn(0), kThreads, resume_smem));
        resume_grid = std::max(1, std::min(n_warp_q, dev_sm * std::max(occ, 1)));
    }
    gstate_mem.reset();
    args.gstate = nullptr;
    args.gstate_stride = block_gs ? (long long)align_up(bp.gst, 256) : 0;
    if (block_gs) {
        CK(cudaMalloc(&gstate_mem.p, (size_t)args.gstate_stride * grid_blocks));
        args.gstate = (unsigned char *)gstate_mem.p;
    }
    // warp-mode plan: as many warps per block as fit in the block's shared
    // memory, at most 16 (128 registers a thread; 64 at level 3), capped by
    // plan.warp_warps.  Placement level as for the blocks (plan.warp_gstate):
    // 1 = a level with at least 1.5x the warps per SM.  Measured on 32,768
    // instances of a 118-bus grid: FP32 level 0 8 warps per SM, warp kernel
    // 8.14 ms; level 2 16 warps per SM, 6.65 ms; FP64 level 0 7 warps per SM
    // 25.3 ms, level 2 8 warps per SM 25.8 ms.
    warp_grid = 0;
    warp_gs = 0;
    size_t warp_gstride = 0;
    if (n_warp_q) {
        struct WarpPlan { int warps = 0, occ = 0; size_t slice = 0, gst = 0; };
        auto plan_warps = [&](int gs, WarpPlan &wp) -> gbpf_status {
            const int lv = std::min(gs, 2);
            for (size_t t = 0; t < topo_h.size(); t++) {
                if (!warp_ok[t]) continue;
                const Topo &T = topo_h[t];
                const Layout w = fp32 ? layout<float>(T.nB, T.n, T.nup, T.nPV, 1, plan.warp_lu1, lv)
                                      : layout<double>(T.nB, T.n, T.nup, T.nPV, 1, plan.warp_lu1, lv);
                wp.slice = std::max(wp.slice, align_up(w.total, 128));
                wp.gst = std::max(wp.gst, w.gtotal);
            }
            wp.warps = (int)std::max<size_t>(1, std::min<size_t>(kWarpsMax, (size_t)maxsm / wp.slice));
            if (plan.warp_warps > 0) wp.warps = std::min(wp.warps, plan.warp_warps);
            const size_t sm = (size_t)wp.warps * wp.slice;
            const void *fn = fp32 ? warp_kernel<float>(gs) : warp_kernel<double>(gs);
            CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&wp.occ, fn, 32 * wp.warps, sm));
            return GBPF_OK;
        };
        WarpPlan wp;
        gbpf_status wst = plan_warps(0, wp);
        if (wst != GBPF_OK) return wst;
        if (plan.warp_gstate) {
            for (int gs = 1; gs <= 3; gs++) {
                WarpPlan c;
                if ((wst = plan_warps(gs, c)) != GBPF_OK) return wst;
                const bool take = plan.warp_gstate >= 2 ? (gs == plan.warp_gstate - 1 && c.occ > 0)
                                                        : 2 * c.occ * c.warps >= 3 * wp.occ * wp.warps;
                if (take) {
                    wp = c;
                    warp_gs = gs;
                }
            }
        }
        slice = wp.slice;
        warp_warps = wp.warps;
        warp_smem = (size_t)warp_warps * slice;
        warp_grid = std::max(1, std::min((n_warp_q + warp_warps - 1) / warp_warps, dev_sm * std::max(wp.occ, 1)));
        warp_gstride = warp_gs ? align_up(wp.gst, 256) : 0;
    }
    warp_gstate_mem.reset();
    if (warp_gs) CK(cudaMalloc(&warp_gstate_mem.p, warp_gstride * (size_t)warp_grid * warp_warps));
    // the shared flat-start iteration of every topology
    flat_mem.reset();
    for (auto &T : topo_h) T.flat = nullptr;
    if (plan.flat_shared) {
        std::vector<size_t> at(topo_h.size(), 0);
        size_t total = 0;
        for (size_t t = 0; t < topo_h.size(); t++) {
            const Topo &T = topo_h[t];
            const int nq = T.n + 2 * T.nup;
            at[t] = total;
            total += fp32 ? flat_layout<float>(T.nB, nq).total : flat_layout<double>(T.nB, nq).total;
        }
        CK(cudaMalloc(&flat_mem.p, total));
        for (size_t t = 0; t < topo_h.size(); t++) {
            Topo &T = topo_h[t];
            const int nq = T.n + 2 * T.nup;
            const FlatLayout F = fp32 ? flat_layout<float>(T.nB, nq) : flat_layout<double>(T.nB, nq);
            char *o = (char *)flat_mem.p + at[t];
            CK(cudaMemcpyAsync(o + F.V0, grids[t].V0.data(), 8 * (size_t)T.nB, cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(o + F.th0, grids[t].theta0.data(), 8 * (size_t)T.nB, cudaMemcpyHostToDevice, stream));
            const size_t fs = align_up((fp32 ? 8 : 16) * (size_t)T.n, 16) + (size_t)T.nB;
            // the warp keeps y and the bus flags in shared memory: beyond the
            // opt-in limit (FP64 past ~13,900 buses) the topology has no shared
            // iteration 0 and its instances compute their own
            if (fs > (size_t)maxsm) continue;
            if (fs > 48 * 1024) {
                if (fp32) CK(cudaFuncSetAttribute(k_flat_start<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fs));
                else CK(cudaFuncSetAttribute(k_flat_start<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fs));
            }
            if (fp32) k_flat_start<float><<<1, 32, fs, stream>>>(T, o, plan.warp_group, plan.quad);
            else k_flat_start<double><<<1, 32, fs, stream>>>(T, o, plan.warp_group, plan.quad);
            CK_LAUNCH();
            T.flat = o;
        }
        CK(cudaStreamSynchronize(stream));
    }
    scratch.reset();
    args.scratch = nullptr;
    args.scratch_stride = (long long)align_up(scr, 256);
    if (scr && grid_blocks) CK(cudaMalloc(&scratch.p, (size_t)args.scratch_stride * grid_blocks));
    args.scratch = (char *)scratch.p;
    if (!counter.p) CK(cudaMalloc(&counter.p, 256));
    topo_d.reset();
    CK(cudaMalloc(&topo_d.p, sizeof(Topo) * topo_h.size()));
    CK(cudaMemcpy(topo_d.p, topo_h.data(), sizeof(Topo) * topo_h.size(), cudaMemcpyHostToDevice));
    args.topo = (const Topo *)topo_d.p;
    args.tol = tol;
    args.max_iter = max_iter;
    args.lim = lim;
    args.ev_cap = ev_cap;
    wargs = args;
    args.counter = (int *)counter.p;
    args.queue = (const int *)queues.p + n_warp_q;
    args.queue_len = n_block_q;
    wargs.counter = (int *)counter.p + 1;
    wargs.flat_on = args.flat_on = (const int *)counter.p + 8;
    wargs.queue = (const int *)queues.p;
    wargs.queue_len = n_warp_q;
    wargs.slice = (int)slice;
    wargs.gstate = (unsigned char *)warp_gstate_mem.p;
    wargs.gstate_stride = (long long)warp_gstride;
    wargs.warp_group = plan.warp_group;
    args.narrow = plan.narrow;
    args.lu1 = plan.lu1;
    args.quad = wargs.quad = plan.quad;
    wargs.lu1 = plan.warp_lu1;
    args.rotate = wargs.rotate = plan.rotate;
    handoff.reset();
    topo_resume.reset();
    wargs.handoff_it = 0;
    if (use_handoff) {
        // a resumed instance whose predicted start failed starts again from
        // the shared iteration 0
        for (size_t t = 0; t < rt.size(); t++) rt[t].flat = topo_h[t].flat;
        CK(cudaMalloc(&topo_resume.p, sizeof(Topo) * rt.size()));
        CK(cudaMemcpy(topo_resume.p, rt.data(), sizeof(Topo) * rt.size(), cudaMemcpyHostToDevice));
        CK(cudaMalloc(&handoff.p, 4 * (size_t)n_warp_q + 256));
        wargs.handoff_it = plan.handoff_it;
        wargs.handoff_q = (int *)handoff.p;
        wargs.handoff_n = (int *)counter.p + 3;
    }
    // one graph: reset the work counter, one persistent launch
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    gbpf_status st = launch(stream);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (st != GBPF_OK) return st;
    if (e != cudaSuccess) { set_error(std::string("capture: ") + cudaGetErrorString(e)); return GBPF_E_CUDA; }
    graph = g;
    CK(cudaGraphInstantiate(&exec, graph, 0));
    return GBPF_OK;
}

// Batched Newton from the learned warm start: features of every instance ->
// network -> per-instance choice between the predicted and the instance's own
// start (initial mismatch) -> one persistent Newton launch from the chosen
// starts -> instances whose predicted start did not converge, or converged far
// from the prediction, are solved again from their own start.  kind[i]: 0 own start chosen up front, 1 predicted
// start converged, 2 predicted start failed and the own start was used.
gbpf_status gbpf_batch::solve_warm(gbpf_mlp *m, int *kind_out, int *witers_out, float *ms) {
    gbpf_status st = warm_launch(m);
    if (st != GBPF_OK) return st;
    return warm_wait(kind_out, witers_out, ms);
}

gbpf_status gbpf_batch::warm_launch(gbpf_mlp *m) {
    if (!exec || n_inst < 1) { set_error("no instances: call gbpf_batch_set_instances first"); return GBPF_E_ARG; }
    if (warm_pending) { set_error("a warm-started solve is in flight: wait for it first"); return GBPF_E_ARG; }
    const gbpf::MlpShape sh = gbpf::mlp_shape(m);
    const int t0 = inst_topo[0];
    const int nB = grids[t0].nB;
    for (int i = 0; i < n_inst; i++)
        if (inst_topo[i] != t0) { set_error("warm start needs every instance on one grid"); return GBPF_E_ARG; }
    if ((sh.n_in != 3 * nB && sh.n_in != 2 * nB) || sh.n_out != 2 * nB) {
        set_error("network shape does not match the grid: inputs must be 3*nB (or 2*nB) and outputs 2*nB");
        return GBPF_E_ARG;
    }
    if (sh.device != device) { set_error("network and batch live on different devices"); return GBPF_E_ARG; }
    if (warm_n != n_inst) {
        warm_mem.reset();
        if (h_kind) { cudaFreeHost(h_kind); h_kind = nullptr; }
        if (h_witers) { cudaFreeHost(h_witers); h_witers = nullptr; }
        const size_t xb = align_up(2 * (size_t)n_inst * sh.kin, 256), pb = align_up(4 * (size_t)n_inst * sh.outp, 256),
                     vb = align_up(8 * (size_t)n_bus_total, 256), ib = align_up(4 * (size_t)n_inst, 256);
        CK(cudaMalloc(&warm_mem.p, xb + pb + 4 * vb + 4 * ib + 8 * kOrderClasses));
        CK(cudaMallocHost(&h_kind, 4 * (size_t)n_inst));
        CK(cudaMallocHost(&h_witers, 4 * (size_t)n_inst));
        char *p = (char *)warm_mem.p;
        wX = (__nv_bfloat16 *)p; wPred = (float *)(p + xb);
        p += xb + pb;
        wV = (double *)p; wTh = (double *)(p + vb); wEF = (float4 *)(p + 2 * vb);
        p += 4 * vb;
        wKind = (int *)p; wQueue = (int *)(p + ib); wIters = (int *)(p + 2 * ib); wCls = (int *)(p + 3 * ib);
        wHist = (int *)(p + 4 * ib);  // class counts, then the order's cursors
        warm_n = n_inst;
    }
    if (!mwork) mwork = gbpf::mlp_work_create();
    gbpf_status st0;
    if (follow_ev) {
        CK(cudaStreamWaitEvent(stream, follow_ev, 0));
        follow_ev = nullptr;
    }
    if ((st0 = make_wref(sh, t0)) != GBPF_OK) return st0;
    CK(cudaEventRecord(ev0, stream));
    CK(cudaMemsetAsync(wHist, 0, 8 * kOrderClasses, stream));
    k_ws_features<<<dim3((sh.kin + 255) / 256, (unsigned)std::min(n_inst, 4096)), 256, 0, stream>>>(
        args.Pliq, args.Qliq, args.V0, args.inst_off, n_inst, nB, sh.n_in, sh.kin, sh.in_mean, sh.in_iscale, wX);
    CK_LAUNCH();
    gbpf_status st = gbpf::mlp_infer(m, wX, n_inst, wPred, stream, mwork);
    if (st != GBPF_OK) return st;
    CK(cudaEventRecord(wev[0], stream));
    {
        // the two starts' phasors in shared memory when the largest grid's fit
        size_t sel = 0;
        for (const Topo &T : topo_h) sel = std::max(sel, 16 * (size_t)T.nB);
        int optin = 0;
        CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
        if (sel <= (size_t)optin) {
            if (sel > 48 * 1024)
                CK(cudaFuncSetAttribute(k_ws_select<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sel));
            k_ws_select<true><<<n_inst, kSelThreads, sel, stream>>>(args, wPred, sh.outp, sh.out_mean, sh.out_scale,
                                                                    wV, wTh, wEF, wKind, wCls, wHist);
        } else {
            k_ws_select<false><<<n_inst, kSelThreads, 0, stream>>>(args, wPred, sh.outp, sh.out_mean, sh.out_scale,
                                                                   wV, wTh, wEF, wKind, wCls, wHist);
        }
    }
    CK_LAUNCH();
    const int order_blocks = std::min((n_inst + 255) / 256, 1024);
    k_ws_order<<<order_blocks, 256, 0, stream>>>(wCls, wHist, wHist + kOrderClasses, n_inst, wQueue);
    CK_LAUNCH();
    CK(cudaEventRecord(wev[1], stream));
    // one launch: predicted starts, own starts, and the restarts of failed
    // predictions, in the order k_ws_order gave
    Args ba = args, wa = wargs;
    for (Args *x : {&ba, &wa}) {
        x->kind = wKind;
        x->witers = wIters;
        x->Vp = wV;
        x->thp = wTh;
        x->warm_max_iter = std::min(max_iter, kWarmMaxIter);
        x->warm_max_dv = kWarmMaxDV;
        x->wref = wref;
    }
    (wa.queue_len ? wa.queue : ba.queue) = wQueue;
    if ((st = launch_with(stream, ba, wa)) != GBPF_OK) return st;
    CK(cudaMemcpyAsync(h_kind, wKind, 4 * (size_t)n_inst, cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(h_witers, wIters, 4 * (size_t)n_inst, cudaMemcpyDeviceToHost, stream));
    CK(cudaEventRecord(ev1, stream));
    CK(cudaEventRecord(step_done, stream));
    warm_pending = true;
    return GBPF_OK;
}

gbpf_status gbpf_batch::make_wref(const gbpf::MlpShape &sh, int t0) {
    std::vector<float> key(sh.h_out_mean, sh.h_out_mean + sh.n_out);
    key.push_back((float)t0);
    key.push_back((float)plan.warp_group);
    if (key == wref_key) return GBPF_OK;
    wref = nullptr;
    wref_key.clear();
    const Topo &T = topo_h[t0];
    const Grid &g = grids[t0];
    const bool fp32 = precision == GBPF_PREC_FP32_IR;
    const int nq = T.n + 2 * T.nup;
    const FlatLayout F = fp32 ? flat_layout<float>(T.nB, nq) : flat_layout<double>(T.nB, nq);
    // k_flat_start's shared memory (y and the bus flags); past the opt-in
    // limit the predicted runs factor their own iteration 0
    const size_t fs = align_up((fp32 ? 8 : 16) * (size_t)T.n, 16) + (size_t)T.nB;
    int maxsm = 0;
    CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    if (fs <= (size_t)maxsm) {
        wref_mem.reset();
        CK(cudaMalloc(&wref_mem.p, F.total));
        wref_h.assign(2 * (size_t)T.nB, 0.0);
        for (int k = 0; k < T.nB; k++) {
            const int ty = g.type[k];
            wref_h[k] = (ty == 0 || ty == 1) ? (double)sh.h_out_mean[k] : g.V0[k];
            wref_h[T.nB + k] = ty == 3 ? g.theta0[k] : (double)sh.h_out_mean[T.nB + k];
        }
        char *o = (char *)wref_mem.p;
        CK(cudaMemcpyAsync(o + F.V0, wref_h.data(), 8 * (size_t)T.nB, cudaMemcpyHostToDevice, stream));
        CK(cudaMemcpyAsync(o + F.th0, wref_h.data() + T.nB, 8 * (size_t)T.nB, cudaMemcpyHostToDevice, stream));
        if (fs > 48 * 1024) {
            if (fp32) CK(cudaFuncSetAttribute(k_flat_start<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fs));
            else CK(cudaFuncSetAttribute(k_flat_start<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fs));
        }
        if (fp32) k_flat_start<float><<<1, 32, fs, stream>>>(T, o, plan.warp_group, plan.quad);
        else k_flat_start<double><<<1, 32, fs, stream>>>(T, o, plan.warp_group, plan.quad);
        CK_LAUNCH();
        wref = o;
    }
    wref_key = key;
    return GBPF_OK;
}

gbpf_status gbpf_batch::warm_wait(int *kind_out, int *witers_out, float *ms) {
    if (!warm_pending) { set_error("no warm-started solve in flight"); return GBPF_E_ARG; }
    warm_pending = false;
    CK(cudaEventSynchronize(ev1));
    if (ms) CK(cudaEventElapsedTime(ms, ev0, ev1));
    CK(cudaEventElapsedTime(&warm_ms[0], ev0, wev[0]));
    CK(cudaEventElapsedTime(&warm_ms[1], wev[0], wev[1]));
    CK(cudaEventElapsedTime(&warm_ms[2], wev[1], ev1));
    if (witers_out)
        for (int i = 0; i < n_inst; i++) witers_out[i] = h_kind[i] ? h_witers[i] : 0;
    if (kind_out) std::copy(h_kind, h_kind + n_inst, kind_out);
    return GBPF_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
#define ARGCHECK(c) do { if (!(c)) { set_error("invalid argument: " #c); return GBPF_E_ARG; } } while (0)

// Coordinate search over the launch plan on the current instances: each knob
// in turn takes each of its values with the others fixed, and a value is kept
// when the whole batch (one graph launch, CUDA events on the batch stream,
// best of `repeats` after one warm-up run) gets at least 2 % faster.  The
// instances' outputs are overwritten by the trial solves; the winning plan
// stays set.  Trial solves of one plan differ from another's only in the
// FP32/FP64 summation order of grouped lanes.
gbpf_status gbpf_batch::autotune(int repeats, float *best_ms, float *first_ms) {
    auto timed = [&](const Plan &p, float *ms) -> gbpf_status {
        plan = p;
        gbpf_status st = rebuild();
        if (st != GBPF_OK) return st;
        CK(cudaGraphLaunch(exec, stream));
        float best = INFINITY;
        for (int r = 0; r < repeats; r++) {
            CK(cudaEventRecord(ev0, stream));
            CK(cudaGraphLaunch(exec, stream));
            CK(cudaEventRecord(ev1, stream));
            CK(cudaEventSynchronize(ev1));
            float t = 0;
            CK(cudaEventElapsedTime(&t, ev0, ev1));
            best = std::min(best, t);
        }
        *ms = best;
        return GBPF_OK;
    };
    // from the default plan (knobs interact: grouping and one-pass levels of
    // the block kernel only matter with a hand-off), two sweeps at most
    Plan cur{};
    float cur_ms = 0;
    gbpf_status st = timed(cur, &cur_ms);
    if (st != GBPF_OK) return st;
    if (first_ms) *first_ms = cur_ms;
    bool any_warp = false;
    for (const Topo &T : topo_h) any_warp |= warp_fits(T);
    bool any_block = false;  // some topology runs on k_nr_block in warp mode too
    for (const Topo &T : topo_h) any_block |= !warp_fits(T);
    struct Knob { int Plan::*field; std::vector<int> values; bool needs_warp, needs_handoff, needs_block; };
    const std::vector<Knob> knobs = {
        {&Plan::warp_mode, {1, 0}, false, false, false},
        {&Plan::warp_group, {1, 0}, true, false, false},
        {&Plan::warp_warps, {8, 0, 6, 4}, true, false, false},
        {&Plan::handoff_it, {kHandoffIt, 6, 8, 16, 24, 0}, true, false, false},
        {&Plan::resume_group, {1, 0}, true, true, false},
        {&Plan::narrow, {1, 0}, false, false, false},
        {&Plan::lu1, {1, 0}, false, false, false},
        {&Plan::warp_lu1, {0, 1}, true, false, false},
        {&Plan::flat_shared, {1, 0}, false, false, false},
        {&Plan::rotate, {0, 1}, false, false, false},
        {&Plan::gstate, {1, 0, 2, 3, 4}, false, false, true},
        {&Plan::warp_gstate, {1, 0, 2, 3, 4}, true, false, false},
    };
    for (int sweep = 0; sweep < 2; sweep++) {
        bool changed = false;
        for (const Knob &k : knobs) {
            if (k.needs_warp && (!any_warp || !cur.warp_mode)) continue;
            if (k.needs_handoff && cur.handoff_it == 0) continue;
            if (k.needs_block && !any_block && cur.warp_mode) continue;
            if (k.field == &Plan::warp_mode && !any_warp) continue;
            const int start = cur.*(k.field);
            for (int v : k.values) {
                if (v == start) continue;
                Plan c = cur;
                c.*(k.field) = v;
                float ms = 0;
                st = timed(c, &ms);
                if (st != GBPF_OK) return st;
                if (ms < 0.98f * cur_ms) { cur = c; cur_ms = ms; changed = true; }
            }
        }
        if (!changed) break;
    }
    // joint trials the one-knob search cannot reach: the 64-register warp
    // kernel (level 3) pays off only with more warps per block than the
    // default, each change alone is slower (118-bus FP32: level 3 with 9
    // warps per block, 18 per SM, 5 % faster than level 2 with 8)
    if (any_warp && cur.warp_mode) {
        for (int w : {9, 10, 12}) {
            Plan c = cur;
            c.warp_gstate = 4;
            c.warp_warps = w;
            float ms = 0;
            st = timed(c, &ms);
            if (st != GBPF_OK) return st;
            if (ms < 0.98f * cur_ms) { cur = c; cur_ms = ms; }
        }
    }
    plan = cur;
    st = rebuild();
    if (best_ms) *best_ms = cur_ms;
    return st;
}

static void plan_out(const gbpf_batch *b, int plan[20]) {
    plan[0] = b->plan.warp_mode;
    plan[1] = b->plan.warp_warps;
    plan[2] = b->plan.handoff_it;
    plan[3] = b->plan.resume_group;
    plan[4] = b->plan.warp_group;
    plan[5] = b->plan.narrow;
    plan[6] = b->plan.lu1;
    plan[7] = b->plan.warp_lu1;
    plan[8] = b->plan.flat_shared;
    plan[9] = b->plan.rotate;
    plan[10] = b->plan.gstate;
    plan[11] = b->plan.warp_gstate;
    plan[12] = b->warp_warps;  // warps per block in use
    plan[13] = b->n_warp_q;
    plan[14] = b->n_block_q;
    plan[15] = b->block_gs;
    plan[16] = b->warp_gs;
    for (int i = 17; i < 20; i++) plan[i] = 0;
}

extern "C" gbpf_status gbpf_batch_get_plan(const gbpf_batch *b, int plan[20]) {
    ARGCHECK(b && plan);
    plan_out(b, plan);
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_set_plan(gbpf_batch *b, const int plan[12]) {
    ARGCHECK(b && plan && (plan[0] == 0 || plan[0] == 1) && plan[1] >= 0 && plan[1] <= kWarpsMax && plan[2] >= 0 &&
             (plan[3] == 0 || plan[3] == 1) && (plan[4] == 0 || plan[4] == 1) && (plan[5] == 0 || plan[5] == 1) &&
             (plan[6] == 0 || plan[6] == 1) && (plan[7] == 0 || plan[7] == 1) && (plan[8] == 0 || plan[8] == 1) &&
             (plan[9] == 0 || plan[9] == 1) && plan[10] >= 0 && plan[10] <= 4 && plan[11] >= 0 && plan[11] <= 4);
    CK(cudaSetDevice(b->device));
    b->plan.warp_mode = plan[0];
    b->plan.warp_warps = plan[1];
    b->plan.handoff_it = plan[2];
    b->plan.resume_group = plan[3];
    b->plan.warp_group = plan[4];
    b->plan.narrow = plan[5];
    b->plan.lu1 = plan[6];
    b->plan.warp_lu1 = plan[7];
    b->plan.flat_shared = plan[8];
    b->plan.rotate = plan[9];
    b->plan.gstate = plan[10];
    b->plan.warp_gstate = plan[11];
    if (!b->n_inst) return GBPF_OK;
    return b->rebuild();
}

extern "C" gbpf_status gbpf_batch_autotune(gbpf_batch *b, int repeats, int plan[20], float ms[2]) {
    ARGCHECK(b && b->exec && repeats > 0);
    CK(cudaSetDevice(b->device));
    float best = 0, first = 0;
    const gbpf_status st = b->autotune(repeats, &best, &first);
    if (st != GBPF_OK) return st;
    if (plan) plan_out(b, plan);
    if (ms) { ms[0] = first; ms[1] = best; }
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_kernel_times(gbpf_batch *b, int repeats, double ms[3]) {
    ARGCHECK(b && b->exec && repeats > 0 && ms);
    CK(cudaSetDevice(b->device));
    ms[0] = ms[1] = ms[2] = 0;
    for (int r = 0; r < repeats; r++) {
        CK(cudaGraphLaunch(b->exec, b->stream));
        CK(cudaStreamSynchronize(b->stream));
        float t = 0;
        if (b->n_block_q) { CK(cudaEventElapsedTime(&t, b->kev[0], b->kev[1])); ms[0] += t; }
        if (b->n_warp_q) {
            CK(cudaEventElapsedTime(&t, b->kev[2], b->kev[3]));
            ms[1] += t;
            if (b->wargs.handoff_it > 0) { CK(cudaEventElapsedTime(&t, b->kev[3], b->kev[4])); ms[2] += t; }
        }
    }
    for (int i = 0; i < 3; i++) ms[i] /= repeats;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_create(const gbpf_grid *const *grids, int n_grids, const gbpf_options *o,
                                         int device, gbpf_batch **out) {
    ARGCHECK(grids && n_grids > 0 && o && out);
    *out = nullptr;
    auto b = std::make_unique<gbpf_batch>();
    b->device = device;
    b->precision = o->precision;
    b->tol = o->tolerancia;
    b->max_iter = o->no_max_iter;
    b->lim = o->lim_inj_reat;
    CK(cudaSetDevice(device));
    {
        const gbpf_status st = trig_table_setup();
        if (st != GBPF_OK) return st;
    }
    CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&b->ev0));
    CK(cudaEventCreate(&b->ev1));
    CK(cudaEventCreateWithFlags(&b->step_done, cudaEventDisableTiming));
    for (auto &e : b->wev) CK(cudaEventCreate(&e));
    for (auto &e : b->pev) CK(cudaEventCreate(&e));
    CK(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming));
    for (auto &e : b->kev) CK(cudaEventCreate(&e));
    for (int i = 0; i < n_grids; i++) {
        ARGCHECK(grids[i]);
        gbpf_status st = b->add_topology(grids[i]->g);
        if (st != GBPF_OK) return st;
    }
    {
        // the grids' own bus values, for instances that do not give theirs
        std::vector<double> dv;
        for (const Grid &g : b->grids) {
            b->dflt_off.push_back((long long)dv.size());
            for (const std::vector<double> *v : {&g.Pload, &g.Qload, &g.Pg, &g.Qg, &g.V0, &g.theta0})
                dv.insert(dv.end(), v->begin(), v->end());
        }
        CK(cudaMalloc(&b->dflt_mem.p, 8 * dv.size()));
        CK(cudaMemcpy(b->dflt_mem.p, dv.data(), 8 * dv.size(), cudaMemcpyHostToDevice));
        CK(cudaMalloc(&b->dflt_off_d.p, 8 * b->dflt_off.size()));
        CK(cudaMemcpy(b->dflt_off_d.p, b->dflt_off.data(), 8 * b->dflt_off.size(), cudaMemcpyHostToDevice));
    }
    // plan for the allocation-free entry point: blobs read from global memory,
    // factors in slices of the static scratch
    {
        const bool fp32 = b->precision == GBPF_PREC_FP32_IR;
        std::vector<Topo> na(b->topo_h);
        for (auto &t : na) {
            t.blob_smem = 0;
            t.fac_smem = 0;
            const Layout l = fp32 ? layout<float>(t.nB, t.n, t.nup, t.nPV, 0, 0) : layout<double>(t.nB, t.n, t.nup, t.nPV, 0, 0);
            b->na_smem.push_back(l.total);
            b->na_stride.push_back(align_up(fp32 ? scratch_bytes<float>(t.n, t.nup) : scratch_bytes<double>(t.n, t.nup),
                                            256));
        }
        CK(cudaMalloc(&b->topo_na.p, sizeof(Topo) * na.size()));
        CK(cudaMemcpy(b->topo_na.p, na.data(), sizeof(Topo) * na.size(), cudaMemcpyHostToDevice));
        void *p = nullptr;
        gbpf_status st = noalloc_setup(device, &p);
        if (st != GBPF_OK) return st;
    }
    *out = b.release();
    return GBPF_OK;
}

// For callers that cannot allocate device memory while they solve (see
// gbpf.h): the batch Newton solve on caller-owned device buffers, with every
// scratch byte in g_noalloc_scratch.  The batch handle is made beforehand with
// gbpf_batch_create (which does allocate, once).  Calls share the scratch, so
// calls that overlap on the GPU race; the work counter is cleared at the start
// of each call and everything else is fully rewritten.  Switch events are not
// recorded.  grid_of_inst is read before the call returns (the per-call
// metadata is staged from it by one copy); the solve itself is asynchronous
// on `stream` (NULL = the batch's own stream).
extern "C" gbpf_status gbpf_batch_solve_noalloc(gbpf_batch *b, int n_inst, const int *grid_of_inst,
                                                const double *V0, const double *theta0, const double *Pliq,
                                                const double *Qliq, const double *Qload, double *V,
                                                double *theta, double *Pcalc, double *Qcalc, int *iterations,
                                                int *status, double *final_mismatch, void *stream) {
    ARGCHECK(b && n_inst > 0 && grid_of_inst && V0 && theta0 && Pliq && Qliq && Qload && V && theta && Pcalc &&
             Qcalc && iterations && status && final_mismatch);
    CK(cudaSetDevice(b->device));
    void *base = nullptr;
    gbpf_status st = noalloc_setup(b->device, &base);
    if (st != GBPF_OK) return st;
    const int nt = (int)b->topo_h.size();
    // per-call metadata: counter | queue | topology ids | bus offsets | event counts | factor slices
    const size_t o_queue = 256, o_topo = o_queue + align_up(4 * (size_t)n_inst, 256),
                 o_off = o_topo + align_up(4 * (size_t)n_inst, 256),
                 o_nev = o_off + align_up(8 * (size_t)n_inst, 256),
                 o_slices = o_nev + align_up(4 * (size_t)n_inst, 256);
    // shared memory and factor slice sized by the grids this call names
    size_t smem = 0, stride = 0;
    for (int i = 0; i < n_inst; i++) {
        const int t = grid_of_inst[i];
        if (t < 0 || t >= nt) { set_error("instance names an unknown grid"); return GBPF_E_ARG; }
        smem = std::max(smem, b->na_smem[t]);
        stride = std::max(stride, b->na_stride[t]);
    }
    int optin = 0;
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device));
    if (smem > (size_t)optin) {
        set_error("gbpf_batch_solve_noalloc: an instance's state needs " + std::to_string(smem >> 10) +
                  " KiB of shared memory; a block holds at most " + std::to_string(optin >> 10) +
                  " KiB (use gbpf_batch_solve for this grid)");
        return GBPF_E_ARG;
    }
    if (o_slices + stride > kNoAllocBytes) {
        set_error("gbpf_batch_solve_noalloc: " + std::to_string(n_inst) + " instances need " +
                  std::to_string((o_slices + stride) >> 10) + " KiB of scratch; the static scratch holds " +
                  std::to_string(kNoAllocBytes >> 10) + " KiB");
        return GBPF_E_ARG;
    }
    // queue | topology ids | bus offsets, laid out as in the scratch, in one
    // host buffer and one copy (a pageable copy: staged before it returns)
    std::vector<unsigned char> meta(o_nev - o_queue);
    int *queue = (int *)meta.data(), *topo = (int *)(meta.data() + (o_topo - o_queue));
    long long *off = (long long *)(meta.data() + (o_off - o_queue));
    long long o = 0;
    for (int i = 0; i < n_inst; i++) {
        queue[i] = i;
        topo[i] = grid_of_inst[i];
        off[i] = o;
        o += b->topo_h[topo[i]].nB;
    }
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    char *sc = (char *)base;
    CK(cudaMemsetAsync(sc, 0, sizeof(int), s));
    CK(cudaMemcpyAsync(sc + o_queue, meta.data(), meta.size(), cudaMemcpyHostToDevice, s));
    Args a{};
    a.topo = (const Topo *)b->topo_na.p;
    a.n_inst = n_inst;
    a.inst_topo = (const int *)(sc + o_topo);
    a.inst_off = (const long long *)(sc + o_off);
    a.V0 = V0; a.th0 = theta0; a.Pliq = Pliq; a.Qliq = Qliq; a.Qload = Qload;
    a.V = V; a.th = theta; a.P = Pcalc; a.Q = Qcalc;
    a.iters = iterations; a.status = status; a.mism = final_mismatch;
    a.n_events = (int *)(sc + o_nev);
    a.events = nullptr;
    a.ev_cap = 0;
    a.tol = b->tol; a.max_iter = b->max_iter; a.lim = b->lim;
    a.counter = (int *)sc;
    a.queue = (const int *)(sc + o_queue);
    a.queue_len = n_inst;
    a.scratch = sc + o_slices;
    a.scratch_stride = (long long)stride;
    a.blob_region = 0;
    const bool fp32 = b->precision == GBPF_PREC_FP32_IR;
    int dev_sm = 0, occ = 0;
    CK(cudaDeviceGetAttribute(&dev_sm, cudaDevAttrMultiProcessorCount, b->device));
    cudaFuncAttributes fa{};
    if (fp32) CK(cudaFuncGetAttributes(&fa, k_nr_block<float, 0>));
    else CK(cudaFuncGetAttributes(&fa, k_nr_block<double, 0>));
    if ((size_t)fa.maxDynamicSharedSizeBytes < smem) {
        const void *fn = fp32 ? (const void *)k_nr_block<float, 0> : (const void *)k_nr_block<double, 0>;
        CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    if (fp32) CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_nr_block<float, 0>, kThreads, smem));
    else CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_nr_block<double, 0>, kThreads, smem));
    const long long slices = (long long)((kNoAllocBytes - o_slices) / stride);
    const int grid = (int)std::max(1LL, std::min<long long>({(long long)n_inst, (long long)dev_sm * std::max(occ, 1), slices}));
    if (fp32) k_nr_block<float, 0><<<grid, kThreads, smem, s>>>(a);
    else k_nr_block<double, 0><<<grid, kThreads, smem, s>>>(a);
    CK_LAUNCH();
    return GBPF_OK;
}

extern "C" void gbpf_batch_free(gbpf_batch *b) { delete b; }

extern "C" gbpf_status gbpf_batch_set_instances(gbpf_batch *b, int n_inst, const int *grid_of_inst,
                                                const double *Pload, const double *Qload, const double *Pg,
                                                const double *Qg, const double *V0, const double *theta0) {
    ARGCHECK(b && n_inst > 0 && grid_of_inst);
    CK(cudaSetDevice(b->device));
    return b->set_instances(n_inst, grid_of_inst, Pload, Qload, Pg, Qg, V0, theta0);
}

extern "C" gbpf_status gbpf_batch_solve(gbpf_batch *b) {
    ARGCHECK(b && b->exec);
    CK(cudaSetDevice(b->device));
    CK(cudaGraphLaunch(b->exec, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_launch(gbpf_batch *b) {
    ARGCHECK(b && b->exec);
    CK(cudaSetDevice(b->device));
    CK(cudaGraphLaunch(b->exec, b->stream));
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_wait(gbpf_batch *b) {
    ARGCHECK(b);
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->stream));
    return GBPF_OK;
}

// `steps` solves spread round-robin over the batches (each on its own
// stream, so one batch's hand-off tail runs beside the next batch's bulk),
// timed with CUDA events: a start event on the first batch's stream that
// every other stream waits for, an end event on each stream, the longest
// span.  All batches must live on one device.
extern "C" gbpf_status gbpf_batch_time_pipelined(gbpf_batch *const *bs, int n, int steps, double *ms) {
    ARGCHECK(bs && n > 0 && steps > 0 && ms);
    for (int i = 0; i < n; i++) ARGCHECK(bs[i] && bs[i]->exec && bs[i]->device == bs[0]->device);
    CK(cudaSetDevice(bs[0]->device));
    for (int i = 0; i < n; i++) CK(cudaStreamSynchronize(bs[i]->stream));
    cudaEvent_t start = bs[0]->ev0;
    CK(cudaEventRecord(start, bs[0]->stream));
    for (int i = 1; i < n; i++) CK(cudaStreamWaitEvent(bs[i]->stream, start, 0));
    for (int k = 0; k < steps; k++) CK(cudaGraphLaunch(bs[k % n]->exec, bs[k % n]->stream));
    float worst = 0;
    for (int i = 0; i < n && i < steps; i++) {
        CK(cudaEventRecord(bs[i]->ev1, bs[i]->stream));
        CK(cudaEventSynchronize(bs[i]->ev1));
        float t = 0;
        CK(cudaEventElapsedTime(&t, start, bs[i]->ev1));
        worst = std::max(worst, t);
    }
    *ms = worst;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_time(gbpf_batch *b, int repeats, double *ms_total) {
    ARGCHECK(b && b->exec && repeats > 0 && ms_total);
    CK(cudaSetDevice(b->device));
    CK(cudaEventRecord(b->ev0, b->stream));
    for (int i = 0; i < repeats; i++) CK(cudaGraphLaunch(b->exec, b->stream));
    CK(cudaEventRecord(b->ev1, b->stream));
    CK(cudaEventSynchronize(b->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    *ms_total = ms;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_results(gbpf_batch *b, int *iterations, int *status, double *final_mismatch,
                                          int *n_events, double *V, double *theta, double *Pcalc, double *Qcalc) {
    ARGCHECK(b && b->n_inst > 0);
    CK(cudaSetDevice(b->device));
    const size_t n = b->n_inst, nb = (size_t)b->n_bus_total * 8;
    // straight into the caller's arrays, one copy each (no staging, no host copy)
    auto down = [&](void *dst, const void *src, size_t bytes) -> gbpf_status {
        if (dst) CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, b->stream));
        return GBPF_OK;
    };
    gbpf_status st;
    if ((st = down(iterations, b->args.iters, 4 * n)) != GBPF_OK) return st;
    if ((st = down(status, b->args.status, 4 * n)) != GBPF_OK) return st;
    if ((st = down(final_mismatch, b->args.mism, 8 * n)) != GBPF_OK) return st;
    if ((st = down(n_events, b->args.n_events, 4 * n)) != GBPF_OK) return st;
    if ((st = down(V, b->args.V, nb)) != GBPF_OK) return st;
    if ((st = down(theta, b->args.th, nb)) != GBPF_OK) return st;
    if ((st = down(Pcalc, b->args.P, nb)) != GBPF_OK) return st;
    if ((st = down(Qcalc, b->args.Q, nb)) != GBPF_OK) return st;
    CK(cudaStreamSynchronize(b->stream));
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_events(gbpf_batch *b, int inst, int *ev, int cap, int *n) {
    ARGCHECK(b && inst >= 0 && inst < b->n_inst && n && (cap == 0 || ev));
    CK(cudaSetDevice(b->device));
    int have = 0;
    CK(cudaMemcpy(&have, b->args.n_events + inst, 4, cudaMemcpyDeviceToHost));
    const int m = std::min(std::min(have, b->ev_cap), cap);
    std::vector<int> e(4 * (size_t)m);
    if (m) CK(cudaMemcpy(e.data(), b->args.events + (size_t)inst * b->ev_cap * 4, e.size() * 4, cudaMemcpyDeviceToHost));
    std::vector<int> idx(m);
    for (int i = 0; i < m; i++) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int x, int y) {
        return e[4 * x] != e[4 * y] ? e[4 * x] < e[4 * y] : e[4 * x + 2] < e[4 * y + 2];
    });
    for (int i = 0; i < m; i++) std::copy(&e[4 * idx[i]], &e[4 * idx[i]] + 4, ev + 4 * i);
    *n = m;
    return have > b->ev_cap ? GBPF_E_ARG : GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_events_all(gbpf_batch *b, int *ev, int cap, int *n) {
    ARGCHECK(b && b->n_inst > 0 && ev && n && cap > 0 && cap <= 16);
    CK(cudaSetDevice(b->device));
    const size_t ni = (size_t)b->n_inst, ec = (size_t)b->ev_cap;
    std::vector<int> e(ni * ec * 4);
    CK(cudaMemcpyAsync(n, b->args.n_events, 4 * ni, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaMemcpyAsync(e.data(), b->args.events, e.size() * 4, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    std::fill(ev, ev + ni * (size_t)cap * 4, 0);
    int idx[16];
    for (size_t i = 0; i < ni; i++) {
        const int *src = e.data() + i * ec * 4;
        const int m = std::min(std::min(n[i], (int)ec), cap);
        for (int k = 0; k < m; k++) idx[k] = k;
        std::sort(idx, idx + m, [&](int x, int y) {
            return src[4 * x] != src[4 * y] ? src[4 * x] < src[4 * y] : src[4 * x + 2] < src[4 * y + 2];
        });
        for (int k = 0; k < m; k++) std::copy(src + 4 * idx[k], src + 4 * idx[k] + 4, ev + (i * cap + k) * 4);
    }
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_solve_warm(gbpf_batch *b, gbpf_mlp *m, int *start_kind, int *warm_iterations,
                                             double *ms) {
    ARGCHECK(b && m);
    CK(cudaSetDevice(b->device));
    float t = 0;
    gbpf_status st = b->solve_warm(m, start_kind, warm_iterations, &t);
    if (ms) *ms = t;
    return st;
}

// `steps` warm-started solves spread round-robin over the batches, each on
// its own stream: a batch whose previous solve is still in flight is waited
// for (on the host) before it is launched again, while the others run.
// Device time from a start event every stream waits for to the last stream's
// end event.
extern "C" gbpf_status gbpf_batch_time_warm_pipelined(gbpf_batch *const *bs, int n, gbpf_mlp *m, int steps,
                                                      double *ms) {
    ARGCHECK(bs && n > 0 && steps > 0 && ms && m);
    for (int i = 0; i < n; i++)
        ARGCHECK(bs[i] && bs[i]->exec && bs[i]->device == bs[0]->device && !bs[i]->warm_pending);
    CK(cudaSetDevice(bs[0]->device));
    for (int i = 0; i < n; i++) CK(cudaStreamSynchronize(bs[i]->stream));
    cudaEvent_t start = bs[0]->pev[0];
    CK(cudaEventRecord(start, bs[0]->stream));
    for (int i = 1; i < n; i++) CK(cudaStreamWaitEvent(bs[i]->stream, start, 0));
    gbpf_status st = GBPF_OK;
    for (int k = 0; k < steps && st == GBPF_OK; k++) {
        gbpf_batch *b = bs[k % n];
        if (b->warm_pending) st = b->warm_wait(nullptr, nullptr, nullptr);
        // each step starts on the device when the previous one has ended: two
        // Newton launches side by side would share the L2 that each one's
        // per-block slices nearly fill (measured: 472-477 k solves/s side by
        // side against 485 k one after the other on the 1,888-bus
        // scenarios); the host still enqueues ahead
        if (st == GBPF_OK && k > 0 && n > 1) b->follow_ev = bs[(k - 1) % n]->step_done;
        if (st == GBPF_OK) st = b->warm_launch(m);
    }
    float worst = 0;
    for (int i = 0; i < n; i++) {
        if (bs[i]->warm_pending) {
            const gbpf_status w = bs[i]->warm_wait(nullptr, nullptr, nullptr);
            if (st == GBPF_OK) st = w;
        }
        if (i >= steps) continue;
        CK(cudaEventRecord(bs[i]->pev[1], bs[i]->stream));
        CK(cudaEventSynchronize(bs[i]->pev[1]));
        float t = 0;
        CK(cudaEventElapsedTime(&t, start, bs[i]->pev[1]));
        worst = std::max(worst, t);
    }
    *ms = worst;
    return st;
}

extern "C" gbpf_status gbpf_batch_follow(gbpf_batch *b, const gbpf_batch *prev) {
    ARGCHECK(b && prev && b != prev && b->device == prev->device);
    b->follow_ev = prev->step_done;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_solve_warm_launch(gbpf_batch *b, gbpf_mlp *m) {
    ARGCHECK(b && m);
    CK(cudaSetDevice(b->device));
    return b->warm_launch(m);
}

extern "C" gbpf_status gbpf_batch_solve_warm_wait(gbpf_batch *b, int *start_kind, int *warm_iterations, double *ms) {
    ARGCHECK(b);
    CK(cudaSetDevice(b->device));
    float t = 0;
    gbpf_status st = b->warm_wait(start_kind, warm_iterations, &t);
    if (ms) *ms = t;
    return st;
}

extern "C" gbpf_status gbpf_batch_warm_phases(const gbpf_batch *b, double ms[3]) {
    ARGCHECK(b && ms);
    for (int i = 0; i < 3; i++) ms[i] = b->warm_ms[i];
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_batch_info(const gbpf_batch *b, long long info[8]) {
    ARGCHECK(b && info);
    long long fs = 0, bs = 0;
    for (auto &t : b->topo_h) { fs += t.fac_smem; bs += t.blob_smem; }
    info[0] = (long long)b->topo_h.size();
    info[1] = b->n_inst;
    info[2] = b->n_bus_total;
    info[3] = b->grid_blocks + b->warp_grid;
    info[4] = (long long)b->smem;
    info[5] = fs;
    info[6] = b->args.scratch_stride;
    info[7] = b->n_warp_q;
    (void)bs;
    return GBPF_OK;
}

// ------------------------------------------------- one-instance solve (solver)
// The single-grid solver's persistent form: a batch of one topology and one
// instance whose block-mode launch reads the solver's start and injections and
// writes the solver's state, events, history and control record in place, so
// that a whole Newton solve is one kernel launch.
struct gbpf::OneSolve {
    gbpf_batch *b = nullptr;
    ~OneSolve() {
        if (b) gbpf_batch_free(b);
    }
};

gbpf_status gbpf::one_create(const Grid &g, const gbpf_options &o, int device, OneSolve **out) {
    *out = nullptr;
    auto s = std::make_unique<OneSolve>();
    gbpf_grid gg{g};
    const gbpf_grid *gp = &gg;
    gbpf_status st = gbpf_batch_create(&gp, 1, &o, device, &s->b);
    if (st != GBPF_OK) return st;
    gbpf_batch *b = s->b;
    // one block, every per-bus array in shared memory, no hand-off, iteration
    // 0 from the shared copy when the start is the grid's.  One-pass levels
    // below 1,000 blocks, two-pass above (measured FP64: 118 buses 0.34 vs
    // 0.38 ms one- vs two-pass; 1,888 buses 1.77 vs 1.61 ms)
    b->plan.warp_mode = 0;
    b->plan.handoff_it = 0;
    b->plan.gstate = 0;
    b->plan.lu1 = g.nB - 1 < 1000 ? 1 : 0;
    b->plan.narrow = 0;
    b->plan.flat_shared = 1;
    const int gi = 0;
    st = b->set_instances(1, &gi, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (st != GBPF_OK) return st;
    if (b->n_block_q != 1 || b->n_warp_q != 0 || b->block_gs != 0 || b->grid_blocks != 1) {
        set_error("one-instance solve: the grid's state does not fit one block's shared memory");
        return GBPF_E_UNSUPPORTED;
    }
    *out = s.release();
    return GBPF_OK;
}

gbpf_status gbpf::one_record(OneSolve *s, void *stream, const OneIO &io) {
    gbpf_batch *b = s->b;
    cudaStream_t st = (cudaStream_t)stream;
    Args a = b->args;
    a.V0 = io.V0; a.th0 = io.th0; a.Pliq = io.Pliq; a.Qliq = io.Qliq; a.Qload = io.Qload;
    a.V = io.V; a.th = io.th; a.P = io.P; a.Q = io.Q;
    a.events = io.events;
    a.ev_cap = io.ev_cap;
    a.hist = io.hist;
    a.trig = io.trig;
    a.hist_cap = io.hist_cap;
    a.limq_out = io.limQ;
    a.ctl_out = io.ctl;
    a.flat_on = io.flat_on;
    a.kind = nullptr;
    CK(cudaMemsetAsync(a.counter, 0, 4 * sizeof(int), st));
    if (b->precision == GBPF_PREC_FP32_IR) k_nr_block<float, 0><<<1, kThreads, b->smem, st>>>(a);
    else k_nr_block<double, 0><<<1, kThreads, b->smem, st>>>(a);
    CK_LAUNCH();
    return GBPF_OK;
}

gbpf_status gbpf::one_set_plan(OneSolve *s, int lu1, int narrow, int quad, int out[3]) {
    gbpf_batch *b = s->b;
    if (lu1 >= 0) b->plan.lu1 = lu1 ? 1 : 0;
    if (narrow >= 0) b->plan.narrow = narrow ? 1 : 0;
    if (quad >= 0) b->plan.quad = quad ? 1 : 0;
    if (lu1 >= 0 || narrow >= 0 || quad >= 0) {
        // the launch arguments and the state layout follow the plan
        CK(cudaSetDevice(b->device));
        gbpf_status st = b->rebuild();
        if (st != GBPF_OK) return st;
        if (b->n_block_q != 1 || b->block_gs != 0 || b->grid_blocks != 1) {
            set_error("one-instance solve: the plan's state does not fit one block's shared memory");
            return GBPF_E_UNSUPPORTED;
        }
    }
    if (out) { out[0] = b->plan.lu1; out[1] = b->plan.narrow; out[2] = b->plan.quad; }
    return GBPF_OK;
}

void gbpf::one_free(OneSolve *s) { delete s; }
