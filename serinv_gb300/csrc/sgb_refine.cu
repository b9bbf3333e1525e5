// y <- alpha * A x + beta * y for a symmetric BTA matrix held by its lower
// stacks (only the lower triangles of the diagonal blocks and of the tip are
// read), and the small kernels of the refined solve.
//
// The product is the residual of iterative refinement (b - A x with the
// original matrix): the symmetric diagonal blocks and the tip go through
// k_symv_blocks, the tip rows' arrow sums through k_arrow_rows, and the
// off-diagonal block products (Lo_{i-1} x_{i-1}, Lo_i^T x_{i+1},
// Ar_i^T x_tip) through one grouped launch of the product engine.
#include <string.h>

#include "sgb_internal.cuh"

namespace sgb {
namespace {

constexpr int kTileRows = 32;
constexpr int kRhs = 8;
constexpr int kThreads = 256;

// One CTA: 32 output rows of block k, up to 8 right-hand sides.  The
// symmetric block is read tile by tile from its lower triangle (tiles above
// the diagonal from their mirror below it), staged in shared memory.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_symv_blocks(const T* __restrict__ Dm, int64_t count, int64_t m, const T* __restrict__ x, int64_t ldx,
                  int64_t xstride, T* __restrict__ y, int64_t ldy, int64_t ystride, int64_t nrhs, T alpha, T beta) {
    __shared__ T S[kTileRows][kTileRows + 1];
    __shared__ T X[kTileRows][kRhs];
    const int64_t tiles = (m + kTileRows - 1) / kTileRows, groups = (nrhs + kRhs - 1) / kRhs;
    const int64_t items = count * tiles * groups;
    const int tid = threadIdx.x;
    const int rr = tid / kRhs, rc = tid % kRhs;  // output row, rhs within the tile
    // work items (block k, row tile, rhs group), strided over the grid
    for (int64_t it = blockIdx.x; it < items; it += gridDim.x) {
    const int64_t k = it / (tiles * groups);
    const int64_t rem = it - k * tiles * groups;
    const int64_t t0 = (rem / groups) * kTileRows;
    const int64_t r0 = (rem % groups) * kRhs;
    const T* D = Dm + k * m * m;
    const T* xk = x + k * xstride;
    T* yk = y + k * ystride;
    T acc = T(0);
    for (int64_t c0 = 0; c0 < m; c0 += kTileRows) {
        __syncthreads();
        for (int e = tid; e < kTileRows * kTileRows; e += kThreads) {
            const int i = e / kTileRows, j = e % kTileRows;
            T v = T(0);
            if (c0 < t0) {  // below the diagonal: D[t0+i][c0+j]
                if (t0 + i < m && c0 + j < m) v = D[(t0 + i) * m + c0 + j];
                S[i][j] = v;
            } else if (c0 > t0) {  // above: mirror of D[c0+i][t0+j]
                if (c0 + i < m && t0 + j < m) v = D[(c0 + i) * m + t0 + j];
                S[j][i] = v;
            } else {  // diagonal tile: lower triangle, mirrored
                const int64_t gi = t0 + i, gj = c0 + j;
                if (gi < m && gj < m && j <= i) v = D[gi * m + gj];
                if (j <= i) {
                    S[i][j] = v;
                    S[j][i] = v;
                }
            }
        }
        for (int e = tid; e < kTileRows * kRhs; e += kThreads) {
            const int i = e / kRhs, r = e % kRhs;
            X[i][r] = (c0 + i < m && r0 + r < nrhs) ? xk[(c0 + i) * ldx + r0 + r] : T(0);
        }
        __syncthreads();
#pragma unroll 8
        for (int j = 0; j < kTileRows; ++j) acc = fma(S[rr][j], X[j][rc], acc);
    }
    const int64_t gr = t0 + rr, gc = r0 + rc;
    if (gr < m && gc < nrhs) {
        T v = alpha * acc;
        if (beta != T(0)) v = fma(beta, yk[gr * ldy + gc], v);
        yk[gr * ldy + gc] = v;
    }
    __syncthreads();  // S and X are refilled by the next item
    }
}

// Tip rows: y_tip[j] += alpha * sum_i Ar_i[j, :] x_i, one CTA per tip row and
// group of 8 right-hand sides, reduced over all blocks.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_arrow_rows(const T* __restrict__ Ar, int64_t n, int64_t a, int64_t b, const T* __restrict__ x, int64_t ldx,
                 T* __restrict__ ytip, int64_t ldy, int64_t nrhs, T alpha) {
    __shared__ T red[kThreads / 32][kRhs];
    const int64_t groups = (nrhs + kRhs - 1) / kRhs;
    // work items (tip row j, rhs group), strided over the grid
    for (int64_t it = blockIdx.x; it < a * groups; it += gridDim.x) {
    const int64_t j = it / groups;
    const int64_t r0 = (it % groups) * kRhs;
    const int nr = (int)((nrhs - r0) < kRhs ? (nrhs - r0) : kRhs);
    T acc[kRhs];
#pragma unroll
    for (int r = 0; r < kRhs; ++r) acc[r] = T(0);
    const int64_t total = n * b;
    for (int64_t e = threadIdx.x; e < total; e += kThreads) {
        const int64_t i = e / b, c = e - i * b;
        const T v = Ar[(i * a + j) * b + c];
        const T* xr = x + e * ldx + r0;
#pragma unroll
        for (int r = 0; r < kRhs; ++r)
            if (r < nr) acc[r] = fma(v, xr[r], acc[r]);
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int r = 0; r < kRhs; ++r) {
        T v = acc[r];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[w][r] = v;
    }
    __syncthreads();
    if (threadIdx.x < nr) {
        T v = T(0);
#pragma unroll
        for (int q = 0; q < kThreads / 32; ++q) v += red[q][threadIdx.x];
        T* yp = ytip + j * ldy + r0 + threadIdx.x;
        *yp = fma(alpha, v, *yp);
    }
    __syncthreads();  // red is refilled by the next item
    }
}

// x += y over rows x cols (leading dimensions ldx, ldy).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_axpy2d(T* __restrict__ x, int64_t ldx, const T* __restrict__ y, int64_t ldy, int64_t rows, int64_t cols) {
    const int64_t total = rows * cols;
    for (int64_t e = blockIdx.x * (int64_t)kThreads + threadIdx.x; e < total; e += (int64_t)gridDim.x * kThreads) {
        const int64_t r = e / cols, c = e - r * cols;
        x[r * ldx + c] += y[r * ldy + c];
    }
}

unsigned grid_1d(int64_t total) {
    int64_t g = (total + kThreads - 1) / kThreads;
    if (g > 152 * 16) g = 152 * 16;
    return (unsigned)(g < 1 ? 1 : g);
}

template <typename T>
GemmProb<T> blank() {
    GemmProb<T> p;
    memset(&p, 0, sizeof(p));
    p.batch = 1;
    return p;
}

template <typename T>
void term(GemmProb<T>& p, int t, const T* A, int64_t lda, int64_t sa, int transA, const T* B, int64_t ldb,
          int64_t sb, int64_t K) {
    p.term[t].A = A;
    p.term[t].lda = lda;
    p.term[t].strideA = sa;
    p.term[t].transA = (int8_t)transA;
    p.term[t].B = B;
    p.term[t].ldb = ldb;
    p.term[t].strideB = sb;
    p.term[t].K = (int32_t)K;
    p.term[t].kmode = KM_FULL;
    if (t + 1 > p.nterms) p.nterms = t + 1;
}

}  // namespace

template <typename T>
cudaError_t bta_symv(const sgb_bta* A, const T* x, int64_t ldx, T* y, int64_t ldy, int64_t nrhs, T alpha, T beta,
                     cudaStream_t s) {
    const int64_t n = A->n, b = A->b, a = A->a;
    if (nrhs <= 0) return cudaSuccess;
    const T* D = (const T*)A->diag;
    const T* Lo = (const T*)A->lower;
    const T* Ar = (const T*)A->arrow;
    const T* Tp = (const T*)A->tip;
    const int64_t groups = (nrhs + kRhs - 1) / kRhs;
    auto grid_items = [](int64_t items) { return (unsigned)(items < 152 * 32 ? items : 152 * 32); };
    // symmetric diagonal blocks and tip (this launch applies beta)
    prof_before(s, SGB_KCLASS_GEMM);
    k_symv_blocks<T><<<grid_items(n * ((b + kTileRows - 1) / kTileRows) * groups), kThreads, 0, s>>>(
        D, n, b, x, ldx, b * ldx, y, ldy, b * ldy, nrhs, alpha, beta);
    prof_after(SGB_KCLASS_GEMM, s, 2.0 * n * b * b * nrhs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (a > 0) {
        prof_before(s, SGB_KCLASS_GEMM);
        k_symv_blocks<T><<<grid_items(((a + kTileRows - 1) / kTileRows) * groups), kThreads, 0, s>>>(
            Tp, 1, a, x + n * b * ldx, ldx, 0, y + n * b * ldy, ldy, 0, nrhs, alpha, beta);
        prof_after(SGB_KCLASS_GEMM, s, 2.0 * a * a * nrhs);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // off-diagonal blocks of the block rows: one grouped launch
    GemmProb<T> pr[3];
    int np = 0;
    const int64_t bb = b * b, ab = a * b, xs = b * ldx, ys = b * ldy;
    const T* xtip = x + n * b * ldx;
    auto row_prob = [&](int64_t i0, int64_t cnt) {
        GemmProb<T> p = blank<T>();
        p.M = (int32_t)b;
        p.N = (int32_t)nrhs;
        p.batch = (int32_t)cnt;
        p.alpha = alpha;
        p.beta = T(1);
        p.Cin = y + i0 * ys;
        p.Cout = y + i0 * ys;
        p.ldcin = p.ldc = ldy;
        p.strideCin = p.strideC = ys;
        return p;
    };
    if (n >= 3) {  // rows 1 .. n-2: Lo_{i-1} x_{i-1} + Lo_i^T x_{i+1} + Ar_i^T x_tip
        GemmProb<T> p = row_prob(1, n - 2);
        term<T>(p, 0, Lo, b, bb, 0, x, ldx, xs, b);
        term<T>(p, 1, Lo + bb, b, bb, 1, x + 2 * xs, ldx, xs, b);
        if (a) term<T>(p, 2, Ar + ab, b, ab, 1, xtip, ldx, 0, a);
        pr[np++] = p;
    }
    if (n >= 2) {
        GemmProb<T> p = row_prob(0, 1);  // row 0: Lo_0^T x_1 + Ar_0^T x_tip
        term<T>(p, 0, Lo, b, 0, 1, x + xs, ldx, 0, b);
        if (a) term<T>(p, 1, Ar, b, 0, 1, xtip, ldx, 0, a);
        pr[np++] = p;
        GemmProb<T> q = row_prob(n - 1, 1);  // row n-1: Lo_{n-2} x_{n-2} + Ar_{n-1}^T x_tip
        term<T>(q, 0, Lo + (n - 2) * bb, b, 0, 0, x + (n - 2) * xs, ldx, 0, b);
        if (a) term<T>(q, 1, Ar + (n - 1) * ab, b, 0, 1, xtip, ldx, 0, a);
        pr[np++] = q;
    } else if (a) {  // n == 1: Ar_0^T x_tip
        GemmProb<T> p = row_prob(0, 1);
        term<T>(p, 0, Ar, b, 0, 1, xtip, ldx, 0, a);
        pr[np++] = p;
    }
    if (np) {
        e = gemm_simt<T>(pr, np, s);
        if (e != cudaSuccess) return e;
    }
    if (a > 0) {  // tip rows: sum_i Ar_i x_i
        prof_before(s, SGB_KCLASS_GEMM);
        k_arrow_rows<T><<<grid_items(a * groups), kThreads, 0, s>>>(Ar, n, a, b, x, ldx, y + n * b * ldy, ldy, nrhs,
                                                                     alpha);
        prof_after(SGB_KCLASS_GEMM, s, 2.0 * a * n * b * nrhs);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename T>
cudaError_t axpy2d(T* x, int64_t ldx, const T* y, int64_t ldy, int64_t rows, int64_t cols, cudaStream_t s) {
    if (rows * cols <= 0) return cudaSuccess;
    prof_before(s, SGB_KCLASS_GEMM);
    k_axpy2d<T><<<grid_1d(rows * cols), kThreads, 0, s>>>(x, ldx, y, ldy, rows, cols);
    prof_after(SGB_KCLASS_GEMM, s, 0.0);
    return cudaGetLastError();
}

template cudaError_t bta_symv<double>(const sgb_bta*, const double*, int64_t, double*, int64_t, int64_t, double,
                                      double, cudaStream_t);
template cudaError_t bta_symv<float>(const sgb_bta*, const float*, int64_t, float*, int64_t, int64_t, float, float,
                                     cudaStream_t);
template cudaError_t axpy2d<double>(double*, int64_t, const double*, int64_t, int64_t, int64_t, cudaStream_t);
template cudaError_t axpy2d<float>(float*, int64_t, const float*, int64_t, int64_t, int64_t, cudaStream_t);

}  // namespace sgb
