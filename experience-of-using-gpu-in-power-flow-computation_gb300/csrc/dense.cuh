// dense.cuh -- the dense linear solve of metodo = denso: the Newton Jacobian as
// a dense FP64 matrix, LU with partial pivoting and the two triangular solves,
// in place of the dense Jacobian kernels (GPU/Jacobiano.cuh:33-222) and the
// cusolverDnXgetrf / getrs calls (GPU/newtonRaphson.cuh:507-530) of the
// reference.  Included by solver.cu after its Dev / Ctl definitions.
//
// The matrix has the sparse path's superset form: 2 x 2 blocks per non-slack
// bus in block order (rows P_j, Q_j; columns theta_j, V_j), a PV bus below its
// limits keeps an identity Q row and a zero V column.  Its solution equals that
// of the reference's reduced system (P rows of the non-slack buses, Q rows of
// the PQ list), so N = 2 (nB - 1) stays fixed while buses switch and the whole
// solve is one static CUDA graph.  Column-major, leading dimension N.
//
// getrf here is right-looking and blocked by kDPanel columns: a one-block panel
// factorisation (pivot = first row of largest magnitude, as LAPACK's idamax),
// the panel's row interchanges applied to the other columns, U12 = L11^-1 A12,
// and the Schur update A22 -= L21 U12 on 64 x 64 FP64 tiles.
#pragma once

constexpr int kDPanel = 32;
constexpr int kDPanelThreads = 1024;
constexpr int kDSolveThreads = 1024;

// Zero the matrix (fill-in positions of a previous pass) and the step's max|dx|.
__global__ void k_dzero(Dev d, int guard) {
    if (stopped(d, guard)) return;
    const long long total = (long long)d.N * d.N / 2;  // N is even
    double2 *A2 = reinterpret_cast<double2 *>(d.A);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x)
        A2[i] = make_double2(0.0, 0.0);
    if (blockIdx.x == 0 && threadIdx.x == 0) d.ctl->maxDx = 0ull;
}

// One thread per bus row: the 2 x 2 blocks of row k (k_jfill's formulas) at
// the dense positions of (block of k, block of m).
__global__ void k_dfill(Dev d, int guard) {
    if (stopped(d, guard)) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.nB || k == d.slack) return;
    const int N = d.N, jr = d.blk_of_bus[k];
    const double Vk = d.V[k];
    const int ak = d.act[k];
    for (int p = d.yptr[k]; p < d.yptr[k + 1]; p++) {
        const int m = d.ycol[p];
        if (m == d.slack) continue;
        const int jc = d.blk_of_bus[m];
        const double2 y = d.yval[p];
        double H, Nn, M, L;
        if (m == k) {
            const double P = d.P[k], Q = d.Q[k], v2 = Vk * Vk;
            H = -Q - v2 * y.y;
            if (ak) { Nn = (P + v2 * y.x) / Vk; M = P - v2 * y.x; L = (Q - v2 * y.y) / Vk; }
            else { Nn = 0.0; M = 0.0; L = 1.0; }
        } else {
            const int am = d.act[m];
            const double ck = d.cs[k], sk = d.sn[k], cm = d.cs[m], sm = d.sn[m];
            const double tr = y.x * cm - y.y * sm, ti = y.x * sm + y.y * cm;
            const double wr = ck * tr + sk * ti, wi = sk * tr - ck * ti;
            const double Vm = d.V[m];
            H = Vk * Vm * wi;
            Nn = am ? Vk * wr : 0.0;
            M = ak ? -Vk * Vm * wr : 0.0;
            L = (ak && am) ? Vk * wi : 0.0;
        }
        double *c0 = d.A + (size_t)(2 * jc) * N, *c1 = c0 + N;
        c0[2 * jr] = H;
        c1[2 * jr] = Nn;
        c0[2 * jr + 1] = M;
        c1[2 * jr + 1] = L;
    }
}

// Panel factorisation of columns k0 .. k0 + nb - 1 over rows k0 .. N - 1, one
// block: for each column the pivot search, the interchange inside the panel,
// the scaling of the column below the pivot and the rank-1 update of the
// panel's remaining columns.  A zero or non-finite pivot ends the solve with
// GBPF_E_SINGULAR.
__global__ void __launch_bounds__(kDPanelThreads) k_dpanel(Dev d, int k0, int guard) {
    if (stopped(d, guard)) return;
    __shared__ double sval[kDPanelThreads / 32];
    __shared__ int sidx[kDPanelThreads / 32];
    __shared__ int spiv;
    const int N = d.N, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb = min(kDPanel, N - k0);
    double *A = d.A;
    for (int jj = 0; jj < nb; jj++) {
        const int j = k0 + jj;
        double *cj = A + (size_t)j * N;
        double best = -1.0;
        int bi = N;
        for (int r = j + tid; r < N; r += kDPanelThreads) {
            double v = fabs(cj[r]);
            if (v != v) v = INFINITY;
            if (v > best) { best = v; bi = r; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) { sval[warp] = best; sidx[warp] = bi; }
        __syncthreads();
        if (tid == 0) {
            double b = sval[0];
            int p = sidx[0];
            for (int w = 1; w < kDPanelThreads / 32; w++)
                if (sval[w] > b || (sval[w] == b && sidx[w] < p)) { b = sval[w]; p = sidx[w]; }
            if (!(b > 0.0) || !isfinite(b) || p >= N) {
                d.ctl->status = GBPF_E_SINGULAR;
                d.ctl->done = 1;
                p = j;
            }
            d.ipiv[j] = p;
            spiv = p;
        }
        __syncthreads();
        const int p = spiv;
        if (p != j)
            for (int c = k0 + tid; c < k0 + nb; c += kDPanelThreads) {
                double *col = A + (size_t)c * N;
                const double t = col[j];
                col[j] = col[p];
                col[p] = t;
            }
        __syncthreads();
        const double pv = cj[j];
        for (int r = j + 1 + tid; r < N; r += kDPanelThreads) cj[r] /= pv;
        __syncthreads();
        for (int c = j + 1; c < k0 + nb; c++) {
            double *col = A + (size_t)c * N;
            const double u = col[j];
            for (int r = j + 1 + tid; r < N; r += kDPanelThreads) col[r] -= cj[r] * u;
        }
        __syncthreads();
    }
}

// The same panel factorisation with the panel (rows k0 .. N-1 of its nb
// columns) in shared memory and one thread per panel row: the pivot search is
// an argmax on the integer order of |a| (NaN counted as +inf, the first row of
// the largest magnitude wins, as idamax), the interchange and the broadcast of
// the pivot row go through one shared buffer, and each thread scales and
// updates its own row with the pivot's reciprocal (as LAPACK's dgetf2 does for
// pivots above the underflow threshold).  Two barriers per column instead of
// four and no FP64 compares.  For panels of at most kDPanelSmemRows rows;
// dynamic shared memory (rows + 1) x nb doubles.
constexpr int kDPanelSmemRows = 832;
__device__ __forceinline__ unsigned long long dabs_key(double v) {
    unsigned long long k = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return k > 0x7ff0000000000000ull ? 0x7ff0000000000000ull : k;  // NaN -> +inf
}
__global__ void __launch_bounds__(kDPanelThreads) k_dpanel_smem(Dev d, int k0, int guard) {
    if (stopped(d, guard)) return;
    extern __shared__ double P[];  // column-major, leading dimension R; then the pivot row (nb)
    __shared__ unsigned long long skey[kDPanelThreads / 32];
    __shared__ int sidx[kDPanelThreads / 32];
    __shared__ int spiv;
    const int N = d.N, R = N - k0, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb = min(kDPanel, R);
    double *A = d.A, *prow = P + (size_t)R * nb;
    for (int i = tid; i < R * nb; i += kDPanelThreads) {
        const int c = i / R, r = i - c * R;
        P[i] = A[(size_t)(k0 + c) * N + k0 + r];
    }
    __syncthreads();
    for (int jj = 0; jj < nb; jj++) {
        // argmax over rows jj..R-1 of column jj
        unsigned long long key = 0;
        int bi = R;
        for (int r = jj + tid; r < R; r += kDPanelThreads) {
            const unsigned long long k = dabs_key(P[(size_t)jj * R + r]);
            if (bi == R || k > key) { key = k; bi = r; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (oi < R && (bi == R || ok > key || (ok == key && oi < bi))) { key = ok; bi = oi; }
        }
        if (lane == 0) { skey[warp] = key; sidx[warp] = bi; }
        __syncthreads();
        if (warp == 0) {
            key = lane < kDPanelThreads / 32 ? skey[lane] : 0;
            bi = lane < kDPanelThreads / 32 ? sidx[lane] : R;
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (oi < R && (bi == R || ok > key || (ok == key && oi < bi))) { key = ok; bi = oi; }
            }
            if (lane == 0) {
                int p = bi;
                if (p >= R || key == 0 || key >= 0x7ff0000000000000ull) {
                    d.ctl->status = GBPF_E_SINGULAR;
                    d.ctl->done = 1;
                    p = jj;
                }
                d.ipiv[k0 + jj] = k0 + p;
                spiv = p;
            }
        }
        // the pivot row into the shared buffer (row p: it becomes row jj)
        __syncthreads();
        const int p = spiv;
        if (tid < nb) prow[tid] = P[(size_t)tid * R + p];
        if (p != jj && tid < nb) P[(size_t)tid * R + p] = P[(size_t)tid * R + jj];
        __syncthreads();
        if (tid < nb) P[(size_t)tid * R + jj] = prow[tid];
        const double inv = 1.0 / prow[jj];
        for (int r = jj + 1 + tid; r < R; r += kDPanelThreads) {
            const double l = P[(size_t)jj * R + r] * inv;
            P[(size_t)jj * R + r] = l;
            for (int c = jj + 1; c < nb; c++) P[(size_t)c * R + r] -= l * prow[c];
        }
        __syncthreads();
    }
    for (int i = tid; i < R * nb; i += kDPanelThreads) {
        const int c = i / R, r = i - c * R;
        A[(size_t)(k0 + c) * N + k0 + r] = P[i];
    }
}

// The panel's interchanges (in order) on every column outside the panel.
__global__ void k_dlaswp(Dev d, int k0, int guard) {
    if (stopped(d, guard)) return;
    const int N = d.N, nb = min(kDPanel, N - k0);
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N || (c >= k0 && c < k0 + nb)) return;
    double *col = d.A + (size_t)c * N;
    for (int j = k0; j < k0 + nb; j++) {
        const int p = d.ipiv[j];
        if (p != j) {
            const double t = col[j];
            col[j] = col[p];
            col[p] = t;
        }
    }
}

// U12 = L11^-1 A12 (L11 unit lower triangular, nb x nb): one thread per column.
__global__ void k_dtrsm(Dev d, int k0, int guard) {
    if (stopped(d, guard)) return;
    __shared__ double L11[kDPanel][kDPanel + 1];
    const int N = d.N, nb = min(kDPanel, N - k0), k1 = k0 + nb;
    for (int i = threadIdx.x; i < nb * nb; i += blockDim.x) {
        const int r = i % nb, t = i / nb;
        L11[r][t] = d.A[(size_t)(k0 + t) * N + k0 + r];
    }
    __syncthreads();
    const int c = k1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    double *col = d.A + (size_t)c * N + k0;
    double x[kDPanel];
#pragma unroll
    for (int i = 0; i < kDPanel; i++) {
        if (i < nb) {
            double v = col[i];
            for (int t = 0; t < i; t++) v -= L11[i][t] * x[t];
            x[i] = v;
            col[i] = v;
        }
    }
}

// A22 -= L21 U12 on 64 x 64 tiles of rows/columns k1 .. N - 1 (K = nb <= 32):
// 256 threads, 4 x 4 outputs each, both operands staged in shared memory.
__global__ void __launch_bounds__(256) k_dgemm(Dev d, int k0, int guard) {
    if (stopped(d, guard)) return;
    __shared__ double Ls[64][kDPanel + 1];
    __shared__ double Us[kDPanel][64 + 1];
    const int N = d.N, nb = min(kDPanel, N - k0), k1 = k0 + nb;
    const int r0 = k1 + blockIdx.y * 64, c0 = k1 + blockIdx.x * 64;
    const int tid = threadIdx.x;
    for (int i = tid; i < 64 * kDPanel; i += 256) {
        const int r = i % 64, t = i / 64;
        Ls[r][t] = (t < nb && r0 + r < N) ? d.A[(size_t)(k0 + t) * N + r0 + r] : 0.0;
    }
    for (int i = tid; i < kDPanel * 64; i += 256) {
        const int t = i % kDPanel, c = i / kDPanel;
        Us[t][c] = (t < nb && c0 + c < N) ? d.A[(size_t)(c0 + c) * N + k0 + t] : 0.0;
    }
    __syncthreads();
    const int tr = (tid / 16) * 4, tc = (tid % 16) * 4;
    double acc[4][4] = {};
    for (int t = 0; t < nb; t++) {
        double a[4], b[4];
#pragma unroll
        for (int q = 0; q < 4; q++) { a[q] = Ls[tr + q][t]; b[q] = Us[t][tc + q]; }
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int s = 0; s < 4; s++) acc[q][s] += a[q] * b[s];
    }
#pragma unroll
    for (int s = 0; s < 4; s++) {
        const int c = c0 + tc + s;
        if (c >= N) continue;
        double *col = d.A + (size_t)c * N;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int r = r0 + tr + q;
            if (r < N) col[r] -= acc[q][s];
        }
    }
}

// getrs: the interchanges on the right-hand side (the mismatch, d.rhs as N
// doubles), L y = b and U x = y in 32-row blocks (the diagonal block by one
// warp, the rest of the rows by the whole block), x into d.xs.  One block; the
// right-hand side lives in dynamic shared memory (8 N bytes).
__global__ void __launch_bounds__(kDSolveThreads) k_dsolve(Dev d, int guard) {
    if (stopped(d, guard)) return;
    extern __shared__ double xsm[];
    __shared__ double blk[32][33];
    const int N = d.N, tid = threadIdx.x, lane = tid & 31;
    const double *b = reinterpret_cast<const double *>(d.rhs);
    for (int i = tid; i < N; i += kDSolveThreads) xsm[i] = b[i];
    __syncthreads();
    if (tid == 0)
        for (int j = 0; j < N; j++) {
            const int p = d.ipiv[j];
            if (p != j) { const double t = xsm[j]; xsm[j] = xsm[p]; xsm[p] = t; }
        }
    __syncthreads();
    const double *A = d.A;
    // forward, unit lower triangular
    for (int jb = 0; jb < N; jb += 32) {
        const int w = min(32, N - jb);
        for (int i = tid; i < w * w; i += kDSolveThreads) blk[i % w][i / w] = A[(size_t)(jb + i / w) * N + jb + i % w];
        __syncthreads();
        if (tid < 32) {
            double x = lane < w ? xsm[jb + lane] : 0.0;
            for (int t = 0; t < w; t++) {
                const double xt = __shfl_sync(0xffffffffu, x, t);
                if (lane > t && lane < w) x -= blk[lane][t] * xt;
            }
            if (lane < w) xsm[jb + lane] = x;
        }
        __syncthreads();
        for (int r = jb + w + tid; r < N; r += kDSolveThreads) {
            double v = xsm[r];
            for (int t = 0; t < w; t++) v -= A[(size_t)(jb + t) * N + r] * xsm[jb + t];
            xsm[r] = v;
        }
        __syncthreads();
    }
    // backward, upper triangular
    for (int je = N; je > 0; je -= 32) {
        const int jb = max(0, je - 32), w = je - jb;
        for (int i = tid; i < w * w; i += kDSolveThreads) blk[i % w][i / w] = A[(size_t)(jb + i / w) * N + jb + i % w];
        __syncthreads();
        if (tid < 32) {
            double x = lane < w ? xsm[jb + lane] : 0.0;
            for (int t = w - 1; t >= 0; t--) {
                if (lane == t) x /= blk[t][t];
                const double xt = __shfl_sync(0xffffffffu, x, t);
                if (lane < t) x -= blk[lane][t] * xt;
            }
            if (lane < w) xsm[jb + lane] = x;
        }
        __syncthreads();
        for (int r = tid; r < jb; r += kDSolveThreads) {
            double v = xsm[r];
            for (int t = 0; t < w; t++) v -= A[(size_t)(jb + t) * N + r] * xsm[jb + t];
            xsm[r] = v;
        }
        __syncthreads();
    }
    for (int j = tid; j < N / 2; j += kDSolveThreads) d.xs[j] = make_double2(xsm[2 * j], xsm[2 * j + 1]);
}
