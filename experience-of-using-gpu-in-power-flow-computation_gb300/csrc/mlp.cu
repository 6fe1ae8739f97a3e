// mlp.cu -- the learned warm start: a dense network
//     features -> hidden (GELU) x n_hidden_layers -> [|V| | theta]
// trained and evaluated by kernels written for sm_103a.  No counterpart in the
// reference (which always starts from v_inicial / theta_inicial,
// GPU/sistInfo.h:62-242); the network only chooses where Newton starts, and
// the Newton loop of batch.cu still decides convergence.
//
// Every matrix product is C[M,N] = A[M,K] * B[N,K]^T with A and B bf16,
// K-contiguous ("K-major"), computed by k_gemm:
//   * one CTA per 128 x 128 output tile, 128 threads;
//   * warp 0 / lane 0 streams 128 x 64 tiles of A and B into a 4-stage
//     shared-memory ring with TMA (cp.async.bulk.tensor, 128-byte swizzle),
//     completion tracked by mbarrier transaction counts;
//   * warp 1 / lane 0 issues tcgen05.mma (kind::f16, bf16 inputs, fp32
//     accumulator 128 x 128 in tensor memory) and frees each stage with
//     tcgen05.commit;
//   * all four warps read the accumulator back with tcgen05.ld (warp w owns
//     TMEM lanes 32w..32w+31 = output rows) and run a fused epilogue.
// Backward products need A^T or B^T; the epilogues that produce an operand
// also write its transpose (coalesced: 32 lanes = 32 consecutive rows).  The
// weight-gradient GEMMs store fp32 gradients; one streaming kernel (k_adam)
// then updates every weight, and k_transpose_bf16 refreshes the transposed
// bf16 copies of the hidden layers' weights.
//
// Every wait on an mbarrier is bounded.  The operand ring's waits take the
// launch's limit (EpiArgs::wait, set per network by gbpf_mlp_set_wait_limit;
// 0 = kWaitCycles); a wait that runs out sets the network's error word, the
// CTA stops issuing work, waits for its tensor-core operations (the
// accumulator barrier) and its copies in flight with the fixed kWaitCycles
// bound, frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "gbpf.h"
#include "gbpf_internal.h"
#include "mlp_internal.h"

using gbpf::set_error;
typedef __nv_bfloat16 bf16;

namespace {

// Three ring stages (96 KB + barriers) so that two CTAs share an SM: one
// CTA's epilogue overlaps the other's main loop, and a 240-tile GEMM runs in
// one wave on 152 SMs (measured with four stages and one CTA per SM: a GEMM
// with a memory-bound epilogue at 17 % of HBM with the tensor pipe 5 % busy)
constexpr int BM = 128, BN = 128, BK = 64, STAGES = 3, kGemmThreads = 128, kGemmCtasPerSm = 2;
constexpr uint32_t kTileBytes = BM * BK * 2;          // 16 KB per operand tile
constexpr uint32_t kStageBytes = 2 * kTileBytes;      // A + B
constexpr size_t kGemmSmem = STAGES * kStageBytes + 1024 + 256;
constexpr long long kWaitCycles = 4000000000ll;       // about 2 s at 2 GHz
// tcgen05 instruction descriptor, kind::f16: fp32 accumulator (bits 4-5 = 1),
// A and B bf16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

enum Epi : int {
    EPI_HIDDEN = 0,      // z = acc + b; Z = z; H = gelu(z); HT = H^T
    EPI_OUT_TRAIN = 1,   // y = acc + b; d = y - target; loss += d^2; H = d * gscale; HT = H^T
    EPI_OUT_INFER = 2,   // out = acc + b
    EPI_BWD_HIDDEN = 3,  // dz = acc * gelu'(Z); H = dz; HT = dz^T
    EPI_WGRAD_STORE = 5, // out = acc (gradient, fp32)
    EPI_OUT_RESID = 6,   // e = acc + b - target; E32 = e; H = bf16(e); loss += lam e^2
    EPI_PROJ = 7,        // r = acc (= (e A)[m, n]); loss += r^2; H = bf16(r)
    EPI_LOSS_GRAD = 8    // q = acc (= (r A^T)[m, n]); H = (q + lam e) * gscale; HT = H^T
};

struct EpiArgs {
    int mode;
    int M, N;             // valid output extent
    int n_real;           // EPI_OUT_TRAIN: columns that carry a loss (the rest are padding)
    int a_row0, b_row0;   // row offsets into the A and B tensor maps
    int a2_row0;          // row offset into the second A map (second operand pair)
    const float *bias;
    float *Z;
    int ldz;
    bf16 *H;
    int ldh;
    bf16 *HT;
    int ldht;
    const float *target;
    int ldt, t_row0;
    float *loss;
    float gscale;
    float lam;            // weight of the plain squared error next to e M e^T
    float *E32;           // residual of the output layer, fp32 [M, lde]
    int lde;
    float *out;
    int ldo;
    int *err;
    long long wait;       // limit of the operand-ring waits in clock cycles (0: kWaitCycles)
    // split-K (training GEMMs with few output tiles): gridDim.z CTAs share an
    // output tile, each over its range of k-tiles; partial tiles go to ws
    // (column-major 128 x 128 fp32 per split) and the last CTA of the tile to
    // arrive (ws_cnt) sums them in split order and runs the epilogue
    float *ws;
    int *ws_cnt;
};

// Learning rate of Adam step t (1-based): cosine decay from lr to sched[2]
// over the sched[1] steps that start after step sched[0].
__device__ __forceinline__ float sched_lr(float lr, const float *sched, int t) {
    const float T = sched[1];
    if (!(T > 0.f)) return lr;
    const float f = fminf(1.f, fmaxf(0.f, ((float)t - sched[0]) / T));
    return sched[2] + 0.5f * (lr - sched[2]) * (1.f + cospif(f));
}

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_test_wait(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase with the given parity to complete, at most
// `limit` clock cycles.  Limits below kPollBelow poll with the non-blocking
// test_wait, so that a short limit runs out when it says (try_wait may
// suspend the thread for a while before it reports an incomplete phase).
constexpr long long kPollBelow = 100000;
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, long long limit = kWaitCycles) {
    if (limit < kPollBelow) {
        const long long t0 = clock64();
        while (!mbar_test_wait(b, parity))
            if (clock64() - t0 > limit) return false;
        return true;
    }
    if (mbar_try_wait(b, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(b, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
// Shared-memory matrix descriptor of a K-major operand tile written by TMA
// with 128-byte swizzle: rows of 128 B, groups of 8 rows 1024 B apart
// (stride byte offset), descriptor version 1 (bits 46-47), layout type
// SWIZZLE_128B (2) in bits 61-63.  The leading byte offset is not used by
// swizzled K-major layouts.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// 8 consecutive fp32 / bf16 values (32 / 16 bytes, aligned: every leading
// dimension and every column group is a multiple of 8 elements)
__device__ __forceinline__ void ld8(const float *p, float (&x)[8]) {
    const float4 a = ((const float4 *)p)[0], b = ((const float4 *)p)[1];
    x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w; x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
}
__device__ __forceinline__ void st8(float *p, const float (&x)[8]) {
    ((float4 *)p)[0] = make_float4(x[0], x[1], x[2], x[3]);
    ((float4 *)p)[1] = make_float4(x[4], x[5], x[6], x[7]);
}
__device__ __forceinline__ void st8h(bf16 *p, const float (&x)[8]) {
    __align__(16) bf16 h[8];
#pragma unroll
    for (int j = 0; j < 8; j++) h[j] = __float2bfloat16_rn(x[j]);
    *(uint4 *)p = *(const uint4 *)h;
}
// transposed bf16 store: 32 lanes = 32 consecutive rows of the transpose
__device__ __forceinline__ void st8t(bf16 *p, int ld, int row, int n, const float (&x)[8]) {
#pragma unroll
    for (int j = 0; j < 8; j++) p[(size_t)(n + j) * ld + row] = __float2bfloat16_rn(x[j]);
}

// Epilogue of 8 accumulator values x = C[row, n .. n+7] (one thread).
__device__ __forceinline__ void epilogue8(const EpiArgs &e, int row, int n, float (&x)[8], float &sq) {
    float b[8], t[8], y[8];
    switch (e.mode) {
    case EPI_HIDDEN:
        ld8(e.bias + n, b);
#pragma unroll
        for (int j = 0; j < 8; j++) { x[j] += b[j]; y[j] = gelu(x[j]); }
        if (e.Z) st8(e.Z + (size_t)row * e.ldz + n, x);
        st8h(e.H + (size_t)row * e.ldh + n, y);
        if (e.HT) st8t(e.HT, e.ldht, row, n, y);
        break;
    case EPI_OUT_TRAIN:
    case EPI_OUT_RESID:
        ld8(e.bias + n, b);
        ld8(e.target + (size_t)(e.t_row0 + row) * e.ldt + n, t);
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float d = n + j < e.n_real ? x[j] + b[j] - t[j] : 0.f;
            if (e.mode == EPI_OUT_TRAIN) {
                sq += d * d;
                y[j] = d * e.gscale;
            } else {
                sq += e.lam * d * d;
                y[j] = d;
            }
        }
        if (e.mode == EPI_OUT_TRAIN) {
            st8h(e.H + (size_t)row * e.ldh + n, y);
            st8t(e.HT, e.ldht, row, n, y);
        } else {
            st8(e.E32 + (size_t)row * e.lde + n, y);
            st8h(e.H + (size_t)row * e.ldh + n, y);
        }
        break;
    case EPI_OUT_INFER:
        ld8(e.bias + n, b);
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] += b[j];
        st8(e.out + (size_t)row * e.ldo + n, x);
        break;
    case EPI_PROJ:
#pragma unroll
        for (int j = 0; j < 8; j++) sq += x[j] * x[j];
        st8h(e.H + (size_t)row * e.ldh + n, x);
        break;
    case EPI_LOSS_GRAD:
        ld8(e.E32 + (size_t)row * e.lde + n, t);
#pragma unroll
        for (int j = 0; j < 8; j++) y[j] = (x[j] + e.lam * t[j]) * e.gscale;
        st8h(e.H + (size_t)row * e.ldh + n, y);
        st8t(e.HT, e.ldht, row, n, y);
        break;
    case EPI_BWD_HIDDEN:
        ld8(e.Z + (size_t)row * e.ldz + n, t);
#pragma unroll
        for (int j = 0; j < 8; j++) y[j] = x[j] * gelu_grad(t[j]);
        st8h(e.H + (size_t)row * e.ldh + n, y);
        st8t(e.HT, e.ldht, row, n, y);
        break;
    default:  // EPI_WGRAD_STORE
        st8(e.out + (size_t)row * e.ldo + n, x);
        break;
    }
}

// ---------------------------------------------------------------------------
// the GEMM
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kGemmThreads, kGemmCtasPerSm)
    k_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
           const __grid_constant__ CUtensorMap ta2, const __grid_constant__ CUtensorMap tb2, int K, int K2,
           EpiArgs e) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + STAGES * kStageBytes);
    uint64_t *empty = full + STAGES;
    uint64_t *accf = empty + STAGES;
    uint32_t *tmem_slot = (uint32_t *)(accf + 1);
    volatile int *fail = (volatile int *)(tmem_slot + 1);
    volatile int *consumed = fail + 1;
    volatile int *issued = fail + 2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    // k-tiles 0..nk1-1 from (ta, tb), then nk2 from (ta2, tb2) into the same
    // accumulator: C = A B^T + A2 B2^T (K2 = 0: one pair)
    const int nk1 = (K + BK - 1) / BK, nk = nk1 + (K2 + BK - 1) / BK;
    const long long wl = e.wait > 0 ? e.wait : kWaitCycles;
    // this CTA's k-tiles [kb, ke) (the whole range unless split)
    const int S = gridDim.z, z = blockIdx.z;
    const int kb = (int)((long long)nk * z / S), ke = (int)((long long)nk * (z + 1) / S);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        mbar_init(accf, 1);
        *fail = 0;
        *consumed = 0;
        *issued = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, BN);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // TMA producer (j counts this CTA's k-tiles: ring slot and phase)
        int j = 0;
        for (; j < ke - kb; j++) {
            const int kt = kb + j, s = j % STAGES;
            if (j >= STAGES && !mbar_wait(&empty[s], ((j / STAGES) - 1) & 1, wl)) { *fail = 1; break; }
            if (*fail) break;
            unsigned char *sa = smem + s * kStageBytes, *sb = sa + kTileBytes;
            mbar_expect_tx(&full[s], kStageBytes);
            if (kt < nk1) {
                tma_load_2d(sa, &ta, kt * BK, e.a_row0 + m0, &full[s]);
                tma_load_2d(sb, &tb, kt * BK, e.b_row0 + n0, &full[s]);
            } else {
                tma_load_2d(sa, &ta2, (kt - nk1) * BK, e.a2_row0 + m0, &full[s]);
                tma_load_2d(sb, &tb2, (kt - nk1) * BK, n0, &full[s]);
            }
        }
        *issued = j;
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        int j = 0;
        for (; j < ke - kb; j++) {
            const int s = j % STAGES;
            if (!mbar_wait(&full[s], (j / STAGES) & 1, wl)) { *fail = 1; break; }
            tc_fence_after();
            const uint32_t sa = smem_u32(smem + s * kStageBytes), sb = sa + kTileBytes;
            const uint64_t da = sw128_desc(sa), db = sw128_desc(sb);
#pragma unroll
            for (int kk = 0; kk < BK / 16; kk++)  // K = 16 per instruction: +32 B along the swizzled row
                mma_bf16(tmem, da + (uint64_t)(2 * kk), db + (uint64_t)(2 * kk), (j | kk) != 0);
            mma_commit(&empty[s]);
        }
        *consumed = j;
        mma_commit(accf);
    }
    __syncwarp();

    // epilogue: warp w reads accumulator rows 32w..32w+31
    const bool ok = mbar_wait(accf, 0);
    tc_fence_after();
    if (!ok) *fail = 1;
    __syncthreads();
    if (*fail) {
        if (threadIdx.x == 0) {
            if (e.err) atomicExch(e.err, 1);
            // copies issued but never consumed are still in flight: wait for them
            for (int j = *consumed; j < *issued; j++) (void)mbar_wait(&full[j % STAGES], (j / STAGES) & 1);
        }
    }
    // split-K: every split stores its partial tile; the last to arrive goes on
    // with the epilogue, the others are done
    __shared__ int s_last;
    const int tile = blockIdx.y * gridDim.x + blockIdx.x;
    const int arow = warp * 32 + lane;  // accumulator row (TMEM lane) of this thread
    if (S > 1 && !*fail) {
        float *part = e.ws + ((size_t)tile * S + z) * BM * BN;
        for (int c = 0; c < BN / 16; c++) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 16), v);
#pragma unroll
            for (int q = 0; q < 16; q++) part[(size_t)(c * 16 + q) * BM + arow] = v[q];
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            s_last = atomicAdd(e.ws_cnt + tile, 1) == S - 1;
            if (s_last) e.ws_cnt[tile] = 0;  // ready for the next GEMM that splits this tile
        }
        __syncthreads();
        __threadfence();
    }
    // the accumulator's 16 columns c*16.. of this thread's row: from tensor
    // memory, or the sum of the splits' partial tiles in split order
    auto acc16 = [&](int c, float (&v)[16]) {
        if (S == 1) {
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 16), v);
            return;
        }
        const float *base = e.ws + (size_t)tile * S * BM * BN + (size_t)(c * 16) * BM + arow;
#pragma unroll
        for (int q = 0; q < 16; q++) v[q] = 0.f;
        for (int zz = 0; zz < S; zz++) {
#pragma unroll
            for (int q = 0; q < 16; q++) v[q] += __ldcg(base + (size_t)zz * BM * BN + (size_t)q * BM);
        }
    };
    if (*fail || (S > 1 && !s_last)) {
        // nothing more to do for this CTA
    } else {
        const int row = m0 + warp * 32 + lane;
        const bool rv = row < e.M;
        float sq = 0.f;
        for (int c = 0; c < BN / 16; c++) {
            const int nb = n0 + c * 16;
            if (nb >= e.N) break;  // uniform across the CTA
            float v[16];
            acc16(c, v);
            if (!rv) continue;
            // N is a multiple of 8: two groups of 8 columns, vector accesses
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (nb + 8 * h >= e.N) break;
                float x[8];
#pragma unroll
                for (int j = 0; j < 8; j++) x[j] = v[8 * h + j];
                epilogue8(e, row, nb + 8 * h, x, sq);
            }
        }
        if (e.mode == EPI_OUT_TRAIN || e.mode == EPI_OUT_RESID || e.mode == EPI_PROJ) {
            for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
            if (lane == 0 && sq != 0.f) atomicAdd(e.loss, sq);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, BN);
}

// ---------------------------------------------------------------------------
// small kernels of a training step
// ---------------------------------------------------------------------------
struct BiasJobs {
    const bf16 *gT[8];  // [rows, cols] transposed pre-activation gradient
    int ld[8], rows[8];
    float *b[8], *bm[8], *bv[8], *gout[8];
    int row_start[9];   // prefix over jobs
    int njobs, cols;
};

// Bias gradient = column sum of dZ over the batch = row sum of dZ^T; then
// Adam on the bias (or store the gradient).  One warp per bias entry.
__global__ void k_bias(BiasJobs J, const int *adam_t, const float *sched, float lr, float b1, float b2, float eps,
                       int adam) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (gw >= J.row_start[J.njobs]) return;
    int j = 0;
    while (gw >= J.row_start[j + 1]) j++;
    const int r = gw - J.row_start[j];
    const bf16 *p = J.gT[j] + (size_t)r * J.ld[j];
    float s = 0.f;
    for (int c = lane; c < J.cols; c += 32) s += __bfloat162float(p[c]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane) return;
    if (!adam) { J.gout[j][r] = s; return; }
    const int ti = *adam_t + 1;
    const float t = (float)ti;
    const float m = b1 * J.bm[j][r] + (1.f - b1) * s, v = b2 * J.bv[j][r] + (1.f - b2) * s * s;
    J.bm[j][r] = m;
    J.bv[j][r] = v;
    J.b[j][r] -= sched_lr(lr, sched, ti) * (m / (1.f - powf(b1, t))) / (sqrtf(v / (1.f - powf(b2, t))) + eps);
}

// Adam on every layer's weights in one streaming pass, after the
// weight-gradient GEMMs stored their fp32 gradients: each weight's gradient,
// master copy and two moments are read once and the master, moments and bf16
// copy written once, four weights a thread and kAdamU groups of them in
// flight (evict-first: 0.8 GB a step for the 1,888-bus network, more than the
// L2).  In the GEMM's epilogue the same update ran tile by tile between main
// loops and reached a third of the HBM bandwidth.
constexpr int kMaxAdamJobs = 9;  // up to 7 hidden layers + the output layer + the skip
struct AdamJobs {
    const float *g[kMaxAdamJobs];
    float *W[kMaxAdamJobs], *m[kMaxAdamJobs], *v[kMaxAdamJobs];
    bf16 *Wb[kMaxAdamJobs];
    long long start[kMaxAdamJobs + 1];  // prefix over the jobs, in groups of four weights
    int njobs;
};
constexpr int kAdamU = 4;

__global__ void __launch_bounds__(256) k_adam(AdamJobs J, const int *adam_t, const float *sched, float lr, float b1,
                                              float b2, float eps) {
    const int ti = *adam_t + 1;
    const float t = (float)ti, lrt = sched_lr(lr, sched, ti);
    const float c1 = 1.f / (1.f - powf(b1, t)), c2 = 1.f / (1.f - powf(b2, t));
    const long long total = J.start[J.njobs], stride = (long long)gridDim.x * blockDim.x;
    for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < total; i0 += stride * kAdamU) {
        float4 g[kAdamU], w[kAdamU], am[kAdamU], av[kAdamU];
        int jb[kAdamU];
        long long o[kAdamU];
#pragma unroll
        for (int u = 0; u < kAdamU; u++) {
            const long long i = i0 + u * stride;
            jb[u] = -1;
            if (i >= total) continue;
            int j = 0;
            while (i >= J.start[j + 1]) j++;
            jb[u] = j;
            o[u] = 4 * (i - J.start[j]);
            g[u] = __ldcs((const float4 *)(J.g[j] + o[u]));
            w[u] = __ldcs((const float4 *)(J.W[j] + o[u]));
            am[u] = __ldcs((const float4 *)(J.m[j] + o[u]));
            av[u] = __ldcs((const float4 *)(J.v[j] + o[u]));
        }
#pragma unroll
        for (int u = 0; u < kAdamU; u++) {
            const int j = jb[u];
            if (j < 0) continue;
            float *wp = &w[u].x, *mp = &am[u].x, *vp = &av[u].x;
            const float *gp = &g[u].x;
            __align__(8) bf16 wb[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                mp[k] = b1 * mp[k] + (1.f - b1) * gp[k];
                vp[k] = b2 * vp[k] + (1.f - b2) * gp[k] * gp[k];
                wp[k] -= lrt * (mp[k] * c1) / (sqrtf(vp[k] * c2) + eps);
                wb[k] = __float2bfloat16_rn(wp[k]);
            }
            __stcs((float4 *)(J.W[j] + o[u]), w[u]);
            __stcs((float4 *)(J.m[j] + o[u]), am[u]);
            __stcs((float4 *)(J.v[j] + o[u]), av[u]);
            __stcs((uint2 *)(J.Wb[j] + o[u]), *(const uint2 *)wb);
        }
    }
}

__global__ void k_step(int *t) { *t += 1; }

// rows of X (bf16, row length a multiple of 8) in the order perm[]
__global__ void k_gather_bf16(const bf16 *X, int ld, const int *perm, int n, bf16 *out) {
    const int per = ld / 8;
    const long long total = (long long)n * per;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long r = i / per, c = i % per;
        ((uint4 *)out)[r * per + c] = ((const uint4 *)X)[(long long)perm[r] * per + c];
    }
}
__global__ void k_gather_f32(const float *Y, int ld, const int *perm, int n, float *out) {
    const int per = ld / 4;
    const long long total = (long long)n * per;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long r = i / per, c = i % per;
        ((float4 *)out)[r * per + c] = ((const float4 *)Y)[(long long)perm[r] * per + c];
    }
}
// XT[(b * kin + k) * B + i] = Xs[(b * B + i) * kin + k]: the transposed
// features of each mini-batch b, for the first layer's weight gradient.
__global__ void k_transpose_batches(const bf16 *Xs, int kin, int B, bf16 *XT) {
    __shared__ bf16 tile[32][33];
    const int b = blockIdx.z, k0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int i = i0 + y, k = k0 + threadIdx.x;
        if (i < B && k < kin) tile[y][threadIdx.x] = Xs[((size_t)b * B + i) * kin + k];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int k = k0 + y, i = i0 + threadIdx.x;
        if (i < B && k < kin) XT[((size_t)b * kin + k) * B + i] = tile[threadIdx.x][y];
    }
}
// Wt [cols, rows] = W^T for bf16 W [rows, cols], through 32 x 32 tiles.
__global__ void k_transpose_bf16(const bf16 *W, int rows, int cols, bf16 *Wt) {
    __shared__ bf16 tile[32][34];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[y][threadIdx.x] = W[(size_t)r * cols + c];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int c = c0 + y, r = r0 + threadIdx.x;
        if (r < rows && c < cols) Wt[(size_t)c * rows + r] = tile[threadIdx.x][y];
    }
}

// bf16 weights and their transpose from the fp32 master weights
__global__ void k_cast_weights(const float *Wm, int out, int in, bf16 *Wb, bf16 *Wt) {
    const long long total = (long long)out * in;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(i / in), c = (int)(i % in);
        const bf16 w = __float2bfloat16_rn(Wm[i]);
        Wb[i] = w;
        Wt[(size_t)c * out + r] = w;
    }
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
#define CK(x)                                                                                      \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess) {                                                                   \
            set_error(std::string(#x) + ": " + cudaGetErrorString(e_));                            \
            return e_ == cudaErrorMemoryAllocation ? GBPF_E_OOM : GBPF_E_CUDA;                     \
        }                                                                                          \
    } while (0)

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

// 2-D bf16 tensor map over a row-major [rows, inner] matrix with leading
// dimension ld (elements), 128 x 64 boxes, 128-byte swizzle, zero fill out of
// bounds (so ragged M, N and K tails contribute zeros).
gbpf_status make_map(CUtensorMap *m, const void *base, int inner, long long rows, int ld) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) { set_error("cuTensorMapEncodeTiled is not available from the driver"); return GBPF_E_CUDA; }
    if (((uintptr_t)base & 15) || (ld * 2) % 16 || inner > ld || rows < 1) {
        set_error("tensor map: base must be 16-byte aligned and rows a multiple of 16 bytes");
        return GBPF_E_ARG;
    }
    cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {BK, BM};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("cuTensorMapEncodeTiled failed: " + std::to_string((int)r)); return GBPF_E_CUDA; }
    return GBPF_OK;
}

// Split-K for GEMMs with fewer output tiles than SMs (the mini-batch GEMMs
// of training, M = batch): S splits per tile with S x tiles <= SMs and at
// least kSplitMinTiles k-tiles per split; only where the caller passes the
// workspace (e.ws, e.ws_cnt: training, one stream).
constexpr int kSplitMax = 8, kSplitMinTiles = 8;
gbpf_status gemm2(cudaStream_t st, const CUtensorMap &ta, const CUtensorMap &tb, const CUtensorMap &ta2,
                  const CUtensorMap &tb2, int M, int N, int K, int K2, const EpiArgs &e) {
    EpiArgs x = e;
    x.M = M;
    x.N = N;
    const int gx = (N + BN - 1) / BN, gy = (M + BM - 1) / BM, tiles = gx * gy;
    const int nk = (K + BK - 1) / BK + (K2 + BK - 1) / BK;
    int S = 1;
    if (x.ws && x.ws_cnt) {
        int dev = 0, sms = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        S = std::max(1, std::min({kSplitMax, sms / tiles, nk / kSplitMinTiles}));
    }
    dim3 grid(gx, gy, S);
    k_gemm<<<grid, kGemmThreads, kGemmSmem, st>>>(ta, tb, ta2, tb2, K, K2, x);
    CK(cudaGetLastError());
    return GBPF_OK;
}
gbpf_status gemm(cudaStream_t st, const CUtensorMap &ta, const CUtensorMap &tb, int M, int N, int K, const EpiArgs &e) {
    return gemm2(st, ta, tb, ta, tb, M, N, K, 0, e);
}

inline size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

inline uint16_t f2bf(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

inline uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
inline double unif(uint64_t &s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

struct Dev {
    void *p = nullptr;
    Dev() = default;
    Dev(const Dev &) = delete;
    Dev &operator=(const Dev &) = delete;
    ~Dev() { if (p) cudaFree(p); }
    void reset() { if (p) cudaFree(p); p = nullptr; }
};

struct Layer {
    int in = 0, out = 0;        // in: padded input width; out: padded output width
    float *Wm, *Am, *Av;        // [out, in]
    bf16 *Wb, *Wt;              // [out, in], [in, out]
    float *b, *bm, *bv;         // [out]
    float *gW, *gb;             // gradients (gradient check only)
    CUtensorMap mW, mWt;
};

// Activations of one batch size.
struct Work {
    int B = 0;
    std::vector<float *> Z;      // [B, out_l] per hidden layer
    std::vector<bf16 *> Hb, HT, dZ, dZT;
    bf16 *dY = nullptr, *dYT = nullptr;
    float *E32 = nullptr;        // output residual (metric loss)
    bf16 *Eb = nullptr, *Rb = nullptr;  // residual, residual x A
    int kp = 0;                  // columns of Rb
    std::vector<CUtensorMap> mH, mHT, mdZ, mdZT;
    CUtensorMap mdY, mdYT, mEb, mRb;
    Dev mem;
};

}  // namespace

struct gbpf_mlp {
    int device = 0;
    int n_in = 0, kin = 0, n_out = 0, outp = 0, hidden = 0, n_hidden = 0;
    int has_skip = 0;  // linear path from the features to the outputs (L.back())
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<Layer> L;
    Dev params, norm, misc;
    // split-K workspace of the training GEMMs: one 128 x 128 fp32 partial per
    // CTA (at most one CTA per SM splits) and one arrival counter per tile
    Dev splitk;
    float *ws = nullptr;
    int *ws_cnt = nullptr;
    std::vector<float> in_mean, in_iscale, out_mean, out_scale;  // host copies
    float *d_in_mean = nullptr, *d_in_iscale = nullptr, *d_out_mean = nullptr, *d_out_scale = nullptr;
    int *d_t = nullptr, *d_err = nullptr;
    long long wait_cycles = 0;  // operand-ring wait limit of every GEMM (0: kWaitCycles)
    float *d_loss = nullptr, *d_sched = nullptr;
    long long steps_done = 0;  // Adam steps taken (host copy of *d_t)
    // data set
    int n_data = 0;
    Dev data;
    bf16 *X = nullptr, *Xs = nullptr, *XT = nullptr;
    float *Y = nullptr, *Ys = nullptr;
    int *perm = nullptr;
    CUtensorMap mXs, mXT;
    // training graph (one epoch)
    Work tw;
    int graph_B = 0, graph_steps = 0;
    cudaGraphExec_t exec = nullptr;
    // inference workspace
    Work iw;
    int iw_cap = 0;
    float lr = 1e-3f;
    float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    // loss metric: loss = (|e A|^2 + lam |e|^2) / (rows * n_out) over the
    // normalised output residual e, A [n_out, k]; without A, plain mean
    // squared error.  Stored as bf16 A [outp, kp] and A^T [kp, outp].
    Dev metric;
    bf16 *Ab = nullptr, *Abt = nullptr;
    int metric_k = 0;  // kp, 0 = no metric
    CUtensorMap mA, mAt;
    float lam = 1.f;

    ~gbpf_mlp() {
        if (exec) cudaGraphExecDestroy(exec);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (stream) cudaStreamDestroy(stream);
    }
    int width(int l) const { return l == 0 ? kin : hidden; }  // input width of layer l
    gbpf_status init(int n_in_, int hidden_, int n_hidden_, int n_out_, int skip, unsigned long long seed, int dev);
    int n_layers() const { return n_hidden + 1; }  // layers of the network proper (without the skip)
    gbpf_status make_work(Work &w, int B, bool train);
    gbpf_status forward(cudaStream_t st, Work &w, const CUtensorMap &mX, int x_row0, int M, const float *target,
                        int t_row0, float *out, bool train);
    gbpf_status backward(cudaStream_t st, Work &w, const CUtensorMap &mXT, int xt_row0, int M, bool adam);
    gbpf_status upload_norm();
};

gbpf_status gbpf_mlp::init(int n_in_, int hidden_, int n_hidden_, int n_out_, int skip, unsigned long long seed,
                           int dev) {
    device = dev;
    has_skip = skip ? 1 : 0;
    n_in = n_in_;
    kin = (n_in + 7) / 8 * 8;
    n_out = n_out_;
    outp = (n_out + 7) / 8 * 8;
    hidden = hidden_;
    n_hidden = n_hidden_;
    CK(cudaSetDevice(device));
    CK(cudaFuncSetAttribute(k_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const int nl = n_hidden + 1, nall = nl + has_skip;
    L.resize(nall);
    size_t bytes = 0;
    for (int l = 0; l < nall; l++) {
        L[l].in = l < nl ? width(l) : kin;
        L[l].out = l >= nl - 1 ? outp : hidden;
        const size_t w = (size_t)L[l].in * L[l].out;
        bytes += 4 * al(4 * w) + 2 * al(2 * w) + 5 * al(4 * (size_t)L[l].out);
    }
    CK(cudaMalloc(&params.p, bytes));
    CK(cudaMemset(params.p, 0, bytes));
    char *p = (char *)params.p;
    auto take = [&](size_t b) { char *r = p; p += al(b); return r; };
    uint64_t s = seed ^ 0x5eed5eedull;
    for (int l = 0; l < nall; l++) {
        Layer &y = L[l];
        const size_t w = (size_t)y.in * y.out;
        y.Wm = (float *)take(4 * w); y.Am = (float *)take(4 * w); y.Av = (float *)take(4 * w);
        y.gW = (float *)take(4 * w);
        y.Wb = (bf16 *)take(2 * w); y.Wt = (bf16 *)take(2 * w);
        y.b = (float *)take(4 * (size_t)y.out); y.bm = (float *)take(4 * (size_t)y.out);
        y.bv = (float *)take(4 * (size_t)y.out); y.gb = (float *)take(4 * (size_t)y.out);
        take(4 * (size_t)y.out);
        // uniform(-a, a) with variance 1 / fan_in over the real inputs; the
        // padded input columns and padded output rows start (and stay) at zero
        const int fan = l == 0 || l == nl ? n_in : y.in, rows = l >= nl - 1 ? n_out : y.out;
        const double a = l == nl ? 0.0 : std::sqrt(3.0 / fan);  // the skip starts at zero
        std::vector<float> hw(w, 0.f);
        for (int r = 0; r < rows; r++)
            for (int c = 0; c < fan; c++) hw[(size_t)r * y.in + c] = (float)((2.0 * unif(s) - 1.0) * a);
        CK(cudaMemcpy(y.Wm, hw.data(), 4 * w, cudaMemcpyHostToDevice));
        k_cast_weights<<<256, 256, 0, stream>>>(y.Wm, y.out, y.in, y.Wb, y.Wt);
        CK(cudaGetLastError());
        gbpf_status st = make_map(&y.mW, y.Wb, y.in, y.out, y.in);
        if (st != GBPF_OK) return st;
        st = make_map(&y.mWt, y.Wt, y.out, y.in, y.out);
        if (st != GBPF_OK) return st;
    }
    CK(cudaMalloc(&norm.p, 2 * al(4 * (size_t)n_in) + 2 * al(4 * (size_t)outp)));
    d_in_mean = (float *)norm.p;
    d_in_iscale = (float *)((char *)norm.p + al(4 * (size_t)n_in));
    d_out_mean = (float *)((char *)norm.p + 2 * al(4 * (size_t)n_in));
    d_out_scale = (float *)((char *)d_out_mean + al(4 * (size_t)outp));
    in_mean.assign(n_in, 0.f);
    in_iscale.assign(n_in, 1.f);
    out_mean.assign(outp, 0.f);
    out_scale.assign(outp, 1.f);
    gbpf_status st = upload_norm();
    if (st != GBPF_OK) return st;
    CK(cudaMalloc(&misc.p, 256));
    CK(cudaMemset(misc.p, 0, 256));
    {
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        const size_t part = (size_t)BM * BN * sizeof(float);
        CK(cudaMalloc(&splitk.p, (size_t)sms * part + 4 * (size_t)sms));
        ws = (float *)splitk.p;
        ws_cnt = (int *)((char *)splitk.p + (size_t)sms * part);
        CK(cudaMemset(ws_cnt, 0, 4 * (size_t)sms));
    }
    d_t = (int *)misc.p;
    d_err = d_t + 1;
    d_loss = (float *)(d_t + 2);
    d_sched = (float *)(d_t + 4);  // 3 floats, zero = constant learning rate
    CK(cudaStreamSynchronize(stream));
    return GBPF_OK;
}

gbpf_status gbpf_mlp::upload_norm() {
    CK(cudaMemcpy(d_in_mean, in_mean.data(), 4 * (size_t)n_in, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_in_iscale, in_iscale.data(), 4 * (size_t)n_in, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_out_mean, out_mean.data(), 4 * (size_t)outp, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_out_scale, out_scale.data(), 4 * (size_t)outp, cudaMemcpyHostToDevice));
    return GBPF_OK;
}

gbpf_status gbpf_mlp::make_work(Work &w, int B, bool train) {
    w.mem.reset();
    w.B = B;
    const int nh = n_hidden;
    size_t bytes = 0;
    const size_t hz = al(4 * (size_t)B * hidden), hb = al(2 * (size_t)B * hidden), yb = al(2 * (size_t)B * outp);
    bytes += nh * hb;
    const size_t ez = al(4 * (size_t)B * outp), rz = al(2 * (size_t)B * std::max(metric_k, 8));
    if (train) bytes += nh * (hz + 3 * hb) + 3 * yb + ez + rz;
    CK(cudaMalloc(&w.mem.p, bytes));
    char *p = (char *)w.mem.p;
    auto take = [&](size_t b) { char *r = p; p += b; return r; };
    w.Z.assign(nh, nullptr); w.Hb.assign(nh, nullptr); w.HT.assign(nh, nullptr);
    w.dZ.assign(nh, nullptr); w.dZT.assign(nh, nullptr);
    w.mH.resize(nh); w.mHT.resize(nh); w.mdZ.resize(nh); w.mdZT.resize(nh);
    for (int l = 0; l < nh; l++) {
        w.Hb[l] = (bf16 *)take(hb);
        gbpf_status st = make_map(&w.mH[l], w.Hb[l], hidden, B, hidden);
        if (st != GBPF_OK) return st;
        if (!train) continue;
        w.Z[l] = (float *)take(hz);
        w.HT[l] = (bf16 *)take(hb);
        w.dZ[l] = (bf16 *)take(hb);
        w.dZT[l] = (bf16 *)take(hb);
        if ((st = make_map(&w.mHT[l], w.HT[l], B, hidden, B)) != GBPF_OK) return st;
        if ((st = make_map(&w.mdZ[l], w.dZ[l], hidden, B, hidden)) != GBPF_OK) return st;
        if ((st = make_map(&w.mdZT[l], w.dZT[l], B, hidden, B)) != GBPF_OK) return st;
    }
    if (train) {
        w.dY = (bf16 *)take(yb);
        w.dYT = (bf16 *)take(yb);
        w.Eb = (bf16 *)take(yb);
        w.E32 = (float *)take(ez);
        w.Rb = (bf16 *)take(rz);
        w.kp = std::max(metric_k, 8);
        gbpf_status st = make_map(&w.mdY, w.dY, outp, B, outp);
        if (st != GBPF_OK) return st;
        if ((st = make_map(&w.mdYT, w.dYT, B, outp, B)) != GBPF_OK) return st;
        if ((st = make_map(&w.mEb, w.Eb, outp, B, outp)) != GBPF_OK) return st;
        if ((st = make_map(&w.mRb, w.Rb, w.kp, B, w.kp)) != GBPF_OK) return st;
    }
    return GBPF_OK;
}

// Forward pass of M rows of the features behind mX (rows x_row0..).  Training:
// hidden layers keep Z, H and H^T, the output layer forms dLoss/dy against
// target rows t_row0.. and accumulates the squared error.  Inference: the
// output layer writes out [M, outp].
gbpf_status gbpf_mlp::forward(cudaStream_t st, Work &w, const CUtensorMap &mX, int x_row0, int M, const float *target,
                              int t_row0, float *out, bool train) {
    const int nl = n_hidden + 1;
    for (int l = 0; l < nl; l++) {
        EpiArgs e{};
        e.err = d_err;
        e.wait = wait_cycles;
        if (train) { e.ws = ws; e.ws_cnt = ws_cnt; }
        e.bias = L[l].b;
        e.a_row0 = l == 0 ? x_row0 : 0;
        const CUtensorMap &ta = l == 0 ? mX : w.mH[l - 1];
        if (l < nl - 1) {
            e.mode = EPI_HIDDEN;
            e.H = w.Hb[l]; e.ldh = hidden;
            if (train) { e.Z = w.Z[l]; e.ldz = hidden; e.HT = w.HT[l]; e.ldht = w.B; }
        } else if (train && Ab) {
            e.mode = EPI_OUT_RESID;
            e.n_real = n_out;
            e.target = target; e.ldt = outp; e.t_row0 = t_row0;
            e.loss = d_loss;
            e.lam = lam;
            e.E32 = w.E32; e.lde = outp;
            e.H = w.Eb; e.ldh = outp;
        } else if (train) {
            e.mode = EPI_OUT_TRAIN;
            e.n_real = n_out;
            e.target = target; e.ldt = outp; e.t_row0 = t_row0;
            e.loss = d_loss;
            e.gscale = 2.f / ((float)M * (float)n_out);
            e.H = w.dY; e.ldh = outp; e.HT = w.dYT; e.ldht = w.B;
        } else {
            e.mode = EPI_OUT_INFER;
            e.out = out; e.ldo = outp;
        }
        gbpf_status s;
        if (l == nl - 1 && has_skip) {
            e.a2_row0 = x_row0;
            s = gemm2(st, ta, L[l].mW, mX, L[nl].mW, M, L[l].out, L[l].in, kin, e);
        } else {
            s = gemm(st, ta, L[l].mW, M, L[l].out, L[l].in, e);
        }
        if (s != GBPF_OK) return s;
    }
    if (train && Ab) {
        // r = e A (loss |r|^2), then dLoss/dy = 2 (r A^T + lam e) / (rows * n_out)
        EpiArgs e{};
        e.err = d_err;
        e.wait = wait_cycles;
        e.ws = ws;
        e.ws_cnt = ws_cnt;
        e.mode = EPI_PROJ;
        e.loss = d_loss;
        e.H = w.Rb; e.ldh = w.kp;
        gbpf_status s = gemm(st, w.mEb, mAt, M, w.kp, outp, e);
        if (s != GBPF_OK) return s;
        EpiArgs g{};
        g.err = d_err;
        g.wait = wait_cycles;
        g.ws = ws;
        g.ws_cnt = ws_cnt;
        g.mode = EPI_LOSS_GRAD;
        g.lam = lam;
        g.gscale = 2.f / ((float)M * (float)n_out);
        g.E32 = w.E32; g.lde = outp;
        g.H = w.dY; g.ldh = outp; g.HT = w.dYT; g.ldht = w.B;
        if ((s = gemm(st, w.mRb, mA, M, outp, w.kp, g)) != GBPF_OK) return s;
    }
    return GBPF_OK;
}

// Backward pass after forward(train): hidden-layer input gradients through the
// transposed weights (before those weights change), then the weight gradient
// of each layer with Adam fused (adam) or stored (gradient check), then the
// biases, then the Adam step counter.
gbpf_status gbpf_mlp::backward(cudaStream_t st, Work &w, const CUtensorMap &mXT, int xt_row0, int M, bool adam) {
    const int nl = n_hidden + 1;
    gbpf_status s;
    for (int l = nl - 1; l >= 0; l--) {
        // gradient w.r.t. this layer's pre-activation is dY (l = nl-1) or dZ[l]
        const CUtensorMap &mG = l == nl - 1 ? w.mdY : w.mdZ[l];
        const CUtensorMap &mGT = l == nl - 1 ? w.mdYT : w.mdZT[l];
        if (l > 0) {
            EpiArgs e{};
            e.err = d_err;
            e.wait = wait_cycles;
            e.ws = ws;
            e.ws_cnt = ws_cnt;
            e.mode = EPI_BWD_HIDDEN;
            e.Z = w.Z[l - 1]; e.ldz = hidden;
            e.H = w.dZ[l - 1]; e.ldh = hidden;
            e.HT = w.dZT[l - 1]; e.ldht = w.B;
            if ((s = gemm(st, mG, L[l].mWt, M, hidden, L[l].out, e)) != GBPF_OK) return s;
        }
        EpiArgs e{};
        e.err = d_err;
        e.wait = wait_cycles;
        e.ws = ws;
        e.ws_cnt = ws_cnt;
        e.b_row0 = l == 0 ? xt_row0 : 0;
        e.mode = EPI_WGRAD_STORE;
        e.out = L[l].gW; e.ldo = L[l].in;
        const CUtensorMap &mIn = l == 0 ? mXT : w.mHT[l - 1];
        if ((s = gemm(st, mGT, mIn, L[l].out, L[l].in, M, e)) != GBPF_OK) return s;
    }
    if (has_skip) {
        // the skip's gradient dY^T X; its transpose is never needed
        Layer &k = L[nl];
        EpiArgs e{};
        e.err = d_err;
        e.wait = wait_cycles;
        e.ws = ws;
        e.ws_cnt = ws_cnt;
        e.b_row0 = xt_row0;
        e.mode = EPI_WGRAD_STORE;
        e.out = k.gW; e.ldo = k.in;
        if ((s = gemm(st, w.mdYT, mXT, k.out, k.in, M, e)) != GBPF_OK) return s;
    }
    if (adam) {
        // every weight gradient is stored (and every input gradient that read
        // the old transposed weights is done): Adam over all weights, then the
        // transposed bf16 copies of the hidden layers' weights
        AdamJobs A{};
        A.njobs = nl + (has_skip ? 1 : 0);
        if (A.njobs > kMaxAdamJobs) { set_error("too many layers for the Adam pass"); return GBPF_E_ARG; }
        A.start[0] = 0;
        for (int j = 0; j < A.njobs; j++) {
            Layer &y = L[j];
            A.g[j] = y.gW; A.W[j] = y.Wm; A.m[j] = y.Am; A.v[j] = y.Av; A.Wb[j] = y.Wb;
            A.start[j + 1] = A.start[j] + (long long)y.out * y.in / 4;
        }
        int dev_sm = 0;
        CK(cudaDeviceGetAttribute(&dev_sm, cudaDevAttrMultiProcessorCount, device));
        const long long groups = A.start[A.njobs];
        const int blocks = (int)std::max(1LL, std::min<long long>(8LL * dev_sm, (groups + 255) / 256));
        k_adam<<<blocks, 256, 0, st>>>(A, d_t, d_sched, lr, b1, b2, eps);
        CK(cudaGetLastError());
        for (int l = 0; l < nl; l++) {
            k_transpose_bf16<<<dim3((L[l].in + 31) / 32, (L[l].out + 31) / 32), dim3(32, 8), 0, st>>>(
                L[l].Wb, L[l].out, L[l].in, L[l].Wt);
            CK(cudaGetLastError());
        }
    }
    BiasJobs J{};
    J.njobs = nl;
    J.cols = M;
    J.row_start[0] = 0;
    for (int l = 0; l < nl; l++) {
        J.gT[l] = l == nl - 1 ? w.dYT : w.dZT[l];
        J.ld[l] = w.B;
        J.rows[l] = L[l].out;
        J.b[l] = L[l].b; J.bm[l] = L[l].bm; J.bv[l] = L[l].bv; J.gout[l] = L[l].gb;
        J.row_start[l + 1] = J.row_start[l] + L[l].out;
    }
    const int warps = J.row_start[nl];
    k_bias<<<(warps * 32 + 255) / 256, 256, 0, st>>>(J, d_t, d_sched, lr, b1, b2, eps, adam ? 1 : 0);
    CK(cudaGetLastError());
    if (adam) {
        k_step<<<1, 1, 0, st>>>(d_t);
        CK(cudaGetLastError());
    }
    return GBPF_OK;
}

namespace gbpf {
MlpShape mlp_shape(const gbpf_mlp *m) {
    MlpShape s;
    s.n_in = m->n_in; s.kin = m->kin; s.n_out = m->n_out; s.outp = m->outp; s.device = m->device;
    s.in_mean = m->d_in_mean; s.in_iscale = m->d_in_iscale; s.out_mean = m->d_out_mean; s.out_scale = m->d_out_scale;
    s.h_out_mean = m->out_mean.data();
    return s;
}

struct MlpWork {
    Work w;
    int cap = 0;
    const gbpf_mlp *net = nullptr;
    int hidden = 0, n_hidden = 0;
};
MlpWork *mlp_work_create() { return new MlpWork(); }
void mlp_work_free(MlpWork *w) { delete w; }

gbpf_status mlp_infer(gbpf_mlp *m, const bf16 *X, int n, float *out, cudaStream_t st, MlpWork *mw) {
    if (n < 1) return GBPF_OK;
    Work &w = mw ? mw->w : m->iw;
    int &cap = mw ? mw->cap : m->iw_cap;
    if (mw && (mw->net != m || mw->hidden != m->hidden || mw->n_hidden != m->n_hidden)) {
        cap = 0;
        mw->net = m;
        mw->hidden = m->hidden;
        mw->n_hidden = m->n_hidden;
    }
    if (n > cap) {
        gbpf_status s = m->make_work(w, n, false);
        if (s != GBPF_OK) return s;
        cap = n;
    }
    CUtensorMap mX;
    gbpf_status s = make_map(&mX, X, m->kin, n, m->kin);
    if (s != GBPF_OK) return s;
    // the hidden-layer maps were made for cap rows: rows n.. are never
    // written in this call and only feed masked output rows
    return m->forward(st, w, mX, 0, n, nullptr, 0, out, false);
}
}  // namespace gbpf

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
#define ARG(c) do { if (!(c)) { set_error("invalid argument: " #c); return GBPF_E_ARG; } } while (0)

namespace {
// The network's error word (set by a GEMM whose wait ran out): read after a
// call's GEMMs and cleared, so that the next call starts clean.
gbpf_status take_err(gbpf_mlp *m) {
    int err = 0;
    CK(cudaMemcpy(&err, m->d_err, 4, cudaMemcpyDeviceToHost));
    if (!err) return GBPF_OK;
    CK(cudaMemset(m->d_err, 0, 4));
    set_error("a tensor-core GEMM wait ran out");
    return GBPF_E_TIMEOUT;
}
}  // namespace

extern "C" gbpf_status gbpf_mlp_set_wait_limit(gbpf_mlp *m, long long cycles) {
    ARG(m && cycles >= 0);
    m->wait_cycles = cycles;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_mlp_create(int n_in, int n_hidden_width, int n_hidden_layers, int n_out,
                                       int linear_skip, unsigned long long seed, int device, gbpf_mlp **out) {
    ARG(out && n_in > 0 && n_out > 0 && n_hidden_layers >= 1 && n_hidden_layers <= 7);
    ARG(n_hidden_width >= 8 && n_hidden_width % 8 == 0);
    *out = nullptr;
    gbpf_mlp *m = new gbpf_mlp();
    gbpf_status st = m->init(n_in, n_hidden_width, n_hidden_layers, n_out, linear_skip, seed, device);
    if (st != GBPF_OK) { delete m; return st; }
    *out = m;
    return GBPF_OK;
}

extern "C" void gbpf_mlp_free(gbpf_mlp *m) { delete m; }

extern "C" gbpf_status gbpf_mlp_set_data(gbpf_mlp *m, const float *X, const float *Y, int n) {
    ARG(m && X && Y && n >= 1);
    CK(cudaSetDevice(m->device));
    // normalisation from the data: per feature mean and standard deviation
    std::vector<double> s1(m->n_in, 0), s2(m->n_in, 0), t1(m->n_out, 0), t2(m->n_out, 0);
    for (int i = 0; i < n; i++) {
        const float *x = X + (size_t)i * m->n_in, *y = Y + (size_t)i * m->n_out;
        for (int k = 0; k < m->n_in; k++) { s1[k] += x[k]; s2[k] += (double)x[k] * x[k]; }
        for (int k = 0; k < m->n_out; k++) { t1[k] += y[k]; t2[k] += (double)y[k] * y[k]; }
    }
    for (int k = 0; k < m->n_in; k++) {
        const double mu = s1[k] / n, var = std::max(0.0, s2[k] / n - mu * mu), sd = std::sqrt(var);
        m->in_mean[k] = (float)mu;
        m->in_iscale[k] = sd > 1e-9 * (std::fabs(mu) + 1.0) ? (float)(1.0 / sd) : 1.f;
    }
    for (int k = 0; k < m->n_out; k++) {
        const double mu = t1[k] / n, var = std::max(0.0, t2[k] / n - mu * mu), sd = std::sqrt(var);
        m->out_mean[k] = (float)mu;
        m->out_scale[k] = sd > 1e-9 * (std::fabs(mu) + 1.0) ? (float)sd : 1.f;
    }
    gbpf_status st = m->upload_norm();
    if (st != GBPF_OK) return st;
    // normalised copies: X as bf16 [n, kin], Y as fp32 [n, outp]
    m->data.reset();
    if (m->exec) { cudaGraphExecDestroy(m->exec); m->exec = nullptr; }
    m->graph_B = 0;
    const size_t xb = al(2 * (size_t)n * m->kin), yb = al(4 * (size_t)n * m->outp);
    CK(cudaMalloc(&m->data.p, 3 * xb + 2 * yb + al(4 * (size_t)n)));
    char *p = (char *)m->data.p;
    m->X = (bf16 *)p; m->Xs = (bf16 *)(p + xb); m->XT = (bf16 *)(p + 2 * xb);
    m->Y = (float *)(p + 3 * xb); m->Ys = (float *)(p + 3 * xb + yb);
    m->perm = (int *)(p + 3 * xb + 2 * yb);
    m->n_data = n;
    const int rows = 4096;
    std::vector<uint16_t> hx((size_t)rows * m->kin);
    std::vector<float> hy((size_t)rows * m->outp);
    for (int r0 = 0; r0 < n; r0 += rows) {
        const int nr = std::min(rows, n - r0);
        for (int i = 0; i < nr; i++) {
            const float *x = X + (size_t)(r0 + i) * m->n_in, *y = Y + (size_t)(r0 + i) * m->n_out;
            uint16_t *dx = hx.data() + (size_t)i * m->kin;
            float *dy = hy.data() + (size_t)i * m->outp;
            for (int k = 0; k < m->kin; k++)
                dx[k] = k < m->n_in ? f2bf((x[k] - m->in_mean[k]) * m->in_iscale[k]) : 0;
            for (int k = 0; k < m->outp; k++) dy[k] = k < m->n_out ? (y[k] - m->out_mean[k]) / m->out_scale[k] : 0.f;
        }
        CK(cudaMemcpy(m->X + (size_t)r0 * m->kin, hx.data(), 2 * (size_t)nr * m->kin, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(m->Y + (size_t)r0 * m->outp, hy.data(), 4 * (size_t)nr * m->outp, cudaMemcpyHostToDevice));
    }
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_mlp_train(gbpf_mlp *m, int epochs, int batch, float lr, float lr_final,
                                      unsigned long long seed, float *epoch_loss, double *ms_total) {
    ARG(m && epochs >= 0 && batch >= 8 && batch % 8 == 0 && lr > 0.f && lr_final >= 0.f);
    ARG(m->n_data >= batch);
    CK(cudaSetDevice(m->device));
    const int n = m->n_data, steps = n / batch;
    m->lr = lr;
    if (!m->exec || m->graph_B != batch) {
        if (m->exec) { cudaGraphExecDestroy(m->exec); m->exec = nullptr; }
        gbpf_status s = m->make_work(m->tw, batch, true);
        if (s != GBPF_OK) return s;
        if ((s = make_map(&m->mXs, m->Xs, m->kin, n, m->kin)) != GBPF_OK) return s;
        if ((s = make_map(&m->mXT, m->XT, batch, (long long)steps * m->kin, batch)) != GBPF_OK) return s;
        // one epoch: shuffle the data set (perm[] is uploaded before each
        // launch), transpose each mini-batch's features, then every step
        CK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
        k_gather_bf16<<<1024, 256, 0, m->stream>>>(m->X, m->kin, m->perm, n, m->Xs);
        k_gather_f32<<<1024, 256, 0, m->stream>>>(m->Y, m->outp, m->perm, n, m->Ys);
        k_transpose_batches<<<dim3((m->kin + 31) / 32, (batch + 31) / 32, steps), dim3(32, 8), 0, m->stream>>>(
            m->Xs, m->kin, batch, m->XT);
        for (int t = 0; t < steps && s == GBPF_OK; t++) {
            s = m->forward(m->stream, m->tw, m->mXs, t * batch, batch, m->Ys, t * batch, nullptr, true);
            if (s == GBPF_OK) s = m->backward(m->stream, m->tw, m->mXT, t * m->kin, batch, true);
        }
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(m->stream, &g);
        if (s != GBPF_OK) { if (g) cudaGraphDestroy(g); return s; }
        if (e != cudaSuccess) { set_error(std::string("capture: ") + cudaGetErrorString(e)); return GBPF_E_CUDA; }
        e = cudaGraphInstantiate(&m->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) { set_error(std::string("instantiate: ") + cudaGetErrorString(e)); return GBPF_E_CUDA; }
        m->graph_B = batch;
        m->graph_steps = steps;
    }
    // the schedule of this call: cosine from lr to lr_final over its steps
    // (lr_final == lr: constant), read by the Adam kernels from the device
    const float sched[3] = {(float)m->steps_done, lr_final == lr ? 0.f : (float)epochs * m->graph_steps, lr_final};
    CK(cudaMemcpyAsync(m->d_sched, sched, sizeof(sched), cudaMemcpyHostToDevice, m->stream));
    CK(cudaMemsetAsync(m->d_err, 0, 4, m->stream));
    uint64_t rs = seed ^ 0xa5a5a5a5ull;
    std::vector<int> perm(n);
    double total = 0;
    for (int ep = 0; ep < epochs; ep++) {
        for (int i = 0; i < n; i++) perm[i] = i;
        for (int i = n - 1; i > 0; i--) std::swap(perm[i], perm[(int)(splitmix(rs) % (uint64_t)(i + 1))]);
        CK(cudaMemcpyAsync(m->perm, perm.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, m->stream));
        CK(cudaMemsetAsync(m->d_loss, 0, 4, m->stream));
        CK(cudaEventRecord(m->e0, m->stream));
        CK(cudaGraphLaunch(m->exec, m->stream));
        CK(cudaEventRecord(m->e1, m->stream));
        float loss = 0, ms = 0;
        CK(cudaMemcpyAsync(&loss, m->d_loss, 4, cudaMemcpyDeviceToHost, m->stream));
        CK(cudaStreamSynchronize(m->stream));
        CK(cudaEventElapsedTime(&ms, m->e0, m->e1));
        total += ms;
        m->steps_done += m->graph_steps;
        { const gbpf_status te = take_err(m); if (te != GBPF_OK) return te; }
        if (epoch_loss) epoch_loss[ep] = loss / ((float)steps * batch * m->n_out);
    }
    if (ms_total) *ms_total = total;
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_mlp_predict(gbpf_mlp *m, const float *X, int n, float *Y) {
    ARG(m && X && Y && n >= 1);
    CK(cudaSetDevice(m->device));
    std::vector<uint16_t> hx((size_t)n * m->kin, 0);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < m->n_in; k++)
            hx[(size_t)i * m->kin + k] = f2bf((X[(size_t)i * m->n_in + k] - m->in_mean[k]) * m->in_iscale[k]);
    Dev buf;
    const size_t xb = al(2 * (size_t)n * m->kin);
    CK(cudaMalloc(&buf.p, xb + 4 * (size_t)n * m->outp));
    CK(cudaMemcpyAsync(buf.p, hx.data(), 2 * (size_t)n * m->kin, cudaMemcpyHostToDevice, m->stream));
    float *out = (float *)((char *)buf.p + xb);
    CK(cudaMemsetAsync(m->d_err, 0, 4, m->stream));
    gbpf_status s = gbpf::mlp_infer(m, (const bf16 *)buf.p, n, out, m->stream);
    if (s != GBPF_OK) return s;
    std::vector<float> hy((size_t)n * m->outp);
    CK(cudaMemcpyAsync(hy.data(), out, 4 * hy.size(), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    { const gbpf_status te = take_err(m); if (te != GBPF_OK) return te; }
    for (int i = 0; i < n; i++)
        for (int k = 0; k < m->n_out; k++)
            Y[(size_t)i * m->n_out + k] = hy[(size_t)i * m->outp + k] * m->out_scale[k] + m->out_mean[k];
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_mlp_gradients(gbpf_mlp *m, const float *Xn, const float *Yn, int n, float *loss,
                                          float *dW, float *db) {
    ARG(m && Xn && Yn && n >= 8 && n % 8 == 0);
    CK(cudaSetDevice(m->device));
    Work w;
    gbpf_status s = m->make_work(w, n, true);
    if (s != GBPF_OK) return s;
    const size_t xb = al(2 * (size_t)n * m->kin);
    Dev buf;
    CK(cudaMalloc(&buf.p, 2 * xb + 4 * (size_t)n * m->outp));
    bf16 *dx = (bf16 *)buf.p, *dxt = (bf16 *)((char *)buf.p + xb);
    float *dy = (float *)((char *)buf.p + 2 * xb);
    std::vector<uint16_t> hx((size_t)n * m->kin, 0), hxt((size_t)n * m->kin, 0);
    std::vector<float> hy((size_t)n * m->outp, 0.f);
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < m->n_in; k++) {
            const uint16_t v = f2bf(Xn[(size_t)i * m->n_in + k]);
            hx[(size_t)i * m->kin + k] = v;
            hxt[(size_t)k * n + i] = v;
        }
        for (int k = 0; k < m->n_out; k++) hy[(size_t)i * m->outp + k] = Yn[(size_t)i * m->n_out + k];
    }
    CK(cudaMemcpy(dx, hx.data(), 2 * hx.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dxt, hxt.data(), 2 * hxt.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dy, hy.data(), 4 * hy.size(), cudaMemcpyHostToDevice));
    CUtensorMap mX, mXT;
    if ((s = make_map(&mX, dx, m->kin, n, m->kin)) != GBPF_OK) return s;
    if ((s = make_map(&mXT, dxt, n, m->kin, n)) != GBPF_OK) return s;
    CK(cudaMemsetAsync(m->d_loss, 0, 4, m->stream));
    CK(cudaMemsetAsync(m->d_err, 0, 4, m->stream));
    if ((s = m->forward(m->stream, w, mX, 0, n, dy, 0, nullptr, true)) != GBPF_OK) return s;
    if ((s = m->backward(m->stream, w, mXT, 0, n, false)) != GBPF_OK) return s;
    float l = 0;
    CK(cudaMemcpyAsync(&l, m->d_loss, 4, cudaMemcpyDeviceToHost, m->stream));
    CK(cudaStreamSynchronize(m->stream));
    { const gbpf_status te = take_err(m); if (te != GBPF_OK) return te; }
    if (loss) *loss = l / ((float)n * m->n_out);
    // gradients of the real (unpadded) parameters, layer after layer
    size_t ow = 0, ob = 0;
    const int nl = m->n_hidden + 1;
    for (int li = 0; li < nl + m->has_skip; li++) {
        const Layer &y = m->L[li];
        const int rows = li >= nl - 1 ? m->n_out : y.out, cols = li == 0 || li == nl ? m->n_in : y.in;
        std::vector<float> g((size_t)y.out * y.in), gb(y.out);
        CK(cudaMemcpy(g.data(), y.gW, 4 * g.size(), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(gb.data(), y.gb, 4 * gb.size(), cudaMemcpyDeviceToHost));
        if (dW)
            for (int r = 0; r < rows; r++)
                std::memcpy(dW + ow + (size_t)r * cols, g.data() + (size_t)r * y.in, 4 * (size_t)cols);
        if (li == nl) break;  // the skip has no bias
        if (db) std::memcpy(db + ob, gb.data(), 4 * (size_t)rows);
        ow += (size_t)rows * cols;
        ob += rows;
    }
    return GBPF_OK;
}

// Parameters of layer `layer` (0 = first): W [rows, cols] row-major and b
// [rows], rows/cols the real (unpadded) sizes.
extern "C" gbpf_status gbpf_mlp_params(gbpf_mlp *m, int layer, float *W, float *b) {
    ARG(m && layer >= 0 && layer <= m->n_hidden + m->has_skip);
    CK(cudaSetDevice(m->device));
    CK(cudaStreamSynchronize(m->stream));
    const Layer &y = m->L[layer];
    const bool sk = layer == m->n_hidden + 1;
    const int rows = layer >= m->n_hidden ? m->n_out : y.out, cols = layer == 0 || sk ? m->n_in : y.in;
    if (sk) b = nullptr;
    if (W) {
        std::vector<float> h((size_t)y.out * y.in);
        CK(cudaMemcpy(h.data(), y.Wm, 4 * h.size(), cudaMemcpyDeviceToHost));
        for (int r = 0; r < rows; r++) std::memcpy(W + (size_t)r * cols, h.data() + (size_t)r * y.in, 4 * (size_t)cols);
    }
    if (b) CK(cudaMemcpy(b, y.b, 4 * (size_t)rows, cudaMemcpyDeviceToHost));
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_mlp_set_params(gbpf_mlp *m, int layer, const float *W, const float *b) {
    ARG(m && layer >= 0 && layer <= m->n_hidden + m->has_skip);
    CK(cudaSetDevice(m->device));
    CK(cudaStreamSynchronize(m->stream));
    Layer &y = m->L[layer];
    const bool sk = layer == m->n_hidden + 1;
    const int rows = layer >= m->n_hidden ? m->n_out : y.out, cols = layer == 0 || sk ? m->n_in : y.in;
    if (sk) b = nullptr;
    if (W) {
        std::vector<float> h((size_t)y.out * y.in, 0.f);
        for (int r = 0; r < rows; r++) std::memcpy(h.data() + (size_t)r * y.in, W + (size_t)r * cols, 4 * (size_t)cols);
        CK(cudaMemcpy(y.Wm, h.data(), 4 * h.size(), cudaMemcpyHostToDevice));
        k_cast_weights<<<256, 256, 0, m->stream>>>(y.Wm, y.out, y.in, y.Wb, y.Wt);
        CK(cudaGetLastError());
    }
    if (b) CK(cudaMemcpy(y.b, b, 4 * (size_t)rows, cudaMemcpyHostToDevice));
    CK(cudaStreamSynchronize(m->stream));
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_mlp_norm(const gbpf_mlp *m, float *in_mean, float *in_scale, float *out_mean,
                                     float *out_scale) {
    ARG(m);
    for (int k = 0; k < m->n_in; k++) {
        if (in_mean) in_mean[k] = m->in_mean[k];
        if (in_scale) in_scale[k] = m->in_iscale[k];
    }
    for (int k = 0; k < m->n_out; k++) {
        if (out_mean) out_mean[k] = m->out_mean[k];
        if (out_scale) out_scale[k] = m->out_scale[k];
    }
    return GBPF_OK;
}

extern "C" gbpf_status gbpf_mlp_set_norm(gbpf_mlp *m, const float *in_mean, const float *in_scale,
                                         const float *out_mean, const float *out_scale) {
    ARG(m && in_mean && in_scale && out_mean && out_scale);
    CK(cudaSetDevice(m->device));
    for (int k = 0; k < m->n_in; k++) { m->in_mean[k] = in_mean[k]; m->in_iscale[k] = in_scale[k]; }
    for (int k = 0; k < m->n_out; k++) { m->out_mean[k] = out_mean[k]; m->out_scale[k] = out_scale[k]; }
    return m->upload_norm();
}

extern "C" gbpf_status gbpf_mlp_set_loss_metric(gbpf_mlp *m, const float *A, int k, float lam) {
    ARG(m && lam >= 0.f && (!A || k >= 1));
    CK(cudaSetDevice(m->device));
    CK(cudaStreamSynchronize(m->stream));
    if (m->exec) { cudaGraphExecDestroy(m->exec); m->exec = nullptr; }
    m->graph_B = 0;
    m->lam = lam;
    m->metric.reset();
    m->Ab = m->Abt = nullptr;
    m->metric_k = 0;
    m->tw.B = 0;
    if (!A) return GBPF_OK;
    const int n = m->n_out, p = m->outp, kp = (k + 7) / 8 * 8;
    std::vector<uint16_t> h((size_t)p * kp, 0), ht((size_t)kp * p, 0);
    for (int r = 0; r < n; r++)
        for (int c = 0; c < k; c++) {
            const uint16_t v = f2bf(A[(size_t)r * k + c]);
            h[(size_t)r * kp + c] = v;
            ht[(size_t)c * p + r] = v;
        }
    CK(cudaMalloc(&m->metric.p, 2 * al(2 * h.size())));
    m->Ab = (bf16 *)m->metric.p;
    m->Abt = (bf16 *)((char *)m->metric.p + al(2 * h.size()));
    CK(cudaMemcpy(m->Ab, h.data(), 2 * h.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m->Abt, ht.data(), 2 * ht.size(), cudaMemcpyHostToDevice));
    m->metric_k = kp;
    gbpf_status st = make_map(&m->mA, m->Ab, kp, p, kp);
    if (st != GBPF_OK) return st;
    return make_map(&m->mAt, m->Abt, p, kp, p);
}

extern "C" gbpf_status gbpf_mlp_dims(const gbpf_mlp *m, int dims[5]) {
    ARG(m && dims);
    dims[0] = m->n_in; dims[1] = m->hidden; dims[2] = m->n_hidden; dims[3] = m->n_out; dims[4] = m->has_skip;
    return GBPF_OK;
}
