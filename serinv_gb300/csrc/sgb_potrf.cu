// Diagonal-tile kernels and the blocked factorizations built on them.
//
// * k_potrf_tile: Cholesky of one <= 32 x 32 diagonal tile in shared
//   memory, plus the tile's triangular inverse (used to turn the panel TRSM
//   into a parallel product), with LAPACK-style pivot reporting.
// * k_trtri_tiles: triangular inverse of the diagonal tiles of many blocks.
// * factor_column_block: right-looking blocked Cholesky of the column block
//   [D_i; Lo_i; Ar_i] — the diagonal block and the rows below it are
//   factored together, tile column by tile column, so the TRSMs of
//   src/serinv/algs/pobtaf.py:120-139 become part of the same sweep.
// * trtri_batched: L^{-1} of many blocks at once (row sweep over tiles).
#include <math.h>
#include <string.h>

#include "sgb_internal.cuh"

namespace sgb {

namespace {

constexpr int NT = 256;

template <typename T>
__device__ __forceinline__ T sgb_rsqrt(T x);
template <>
__device__ __forceinline__ double sgb_rsqrt<double>(double x) { return rsqrt(x); }
template <>
__device__ __forceinline__ float sgb_rsqrt<float>(float x) { return rsqrtf(x); }

// Inverse of the lower-triangular tile s (32 x 32, identity-padded beyond
// nb) into x, given the reciprocal diagonal yv.  Recursive doubling keeps
// every step a small parallel product, so no thread runs a long dependent
// chain of FP64 operations (each FP64 warp instruction costs ~64 issue
// cycles on this part):
//   leaves: the four 8 x 8 diagonal blocks by forward substitution;
//   level 1: X21 = -X22 (L21 X11) for the two 16 x 16 blocks;
//   level 2: the same for the 32 x 32 tile.
// Requires all NT threads; ends with a barrier.
template <typename T>
__device__ __forceinline__ void tile_inverse(T (*s)[kTile + 1], T (*x)[kTile + 1], T (*tmp)[kTile + 1],
                                             const T* yv) {
    const int tid = threadIdx.x;
    for (int e = tid; e < kTile * kTile; e += NT) x[e / kTile][e % kTile] = T(0);
    __syncthreads();
    if (tid < 32) {  // leaves: 4 blocks x 8 columns
        const int blk = tid >> 3, jj = tid & 7, b0 = blk * 8, j = b0 + jj;
        for (int r = j; r < b0 + 8; ++r) {
            T sum = (r == j) ? T(1) : T(0);
            for (int k = j; k < r; ++k) sum = fma(-s[r][k], x[k][j], sum);
            x[r][j] = sum * yv[r];
        }
    }
    __syncthreads();
#pragma unroll 1
    for (int h = 8; h < kTile; h *= 2) {  // block size h -> 2h
        const int nblk = kTile / (2 * h);
        // tmp = L21 X11 for every 2h-block (h x h each)
        for (int e = tid; e < nblk * h * h; e += NT) {
            const int bi = e / (h * h), rem = e % (h * h), r = rem / h, c = rem % h;
            const int o = bi * 2 * h;
            T sum = T(0);
            for (int k = c; k < h; ++k) sum = fma(s[o + h + r][o + k], x[o + k][o + c], sum);
            tmp[o + h + r][o + c] = sum;
        }
        __syncthreads();
        // X21 = -X22 tmp
        for (int e = tid; e < nblk * h * h; e += NT) {
            const int bi = e / (h * h), rem = e % (h * h), r = rem / h, c = rem % h;
            const int o = bi * 2 * h;
            T sum = T(0);
            for (int k = 0; k <= r; ++k) sum = fma(x[o + h + r][o + h + k], tmp[o + h + k][o + c], sum);
            x[o + h + r][o + c] = -sum;
        }
        __syncthreads();
    }
}

// Cholesky of one <= 32 x 32 diagonal tile plus its inverse, with a
// one-column lookahead.  Warp 0 (alone on its SM quarter, so nothing else
// competes for that quarter's FP64 unit) owns the pivot chain: per column j
// it forms 1/sqrt(d_j), scales column j, and after the barrier applies
// column j to column j+1 only, so the next pivot is ready.  Warps on the
// other three quarters (1-3, 5-7) meanwhile apply column j-1 to columns
// j+1.. of the trailing triangle.  One barrier per column; the dependent
// FP64 chain per column is rsqrt + one multiply + one FMA.
template <typename T>
__global__ void __launch_bounds__(NT)
k_potrf_tile(T* A, int64_t ld, int nb, int zero_right, T* tinv, int32_t* info, int64_t row0) {
    __shared__ T s[kTile][kTile + 1];
    __shared__ T x[kTile][kTile + 1];
    __shared__ T tmp[kTile][kTile + 1];
    __shared__ T yv[kTile];
    __shared__ int fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int e = tid; e < kTile * kTile; e += NT) {
        const int r = e / kTile, c = e % kTile;
        T v = T(0);
        if (r < nb && c <= r) v = A[(int64_t)r * ld + c];
        else if (r >= nb && r == c) v = T(1);  // identity padding
        s[r][c] = v;
    }
    if (tid == 0) fail = 0;
    if (tid < kTile) yv[tid] = T(1);
    __syncthreads();

    // update workers: warps 1,2,3,5,6,7 -> worker index 0..5
    const int wk = warp == 0 || warp == 4 ? -1 : (warp < 4 ? warp - 1 : warp - 2);
    const int nworkers = 6 * 32;
    for (int j = 0; j < nb; ++j) {
        if (warp == 0) {
            const T d = s[j][j];
            const bool bad = !(d > T(0)) || !isfinite((double)d);
            const T y = bad ? T(NAN) : sgb_rsqrt<T>(d);
            const int r = lane;
            if (r > j && r < nb) s[r][j] *= y;
            if (r == j) {
                s[j][j] = d * y;
                yv[j] = y;
                if (bad && fail == 0) fail = j + 1;
            }
        } else if (wk >= 0 && j >= 1) {
            // column j-1 applied to columns j+1 .. nb-1 (column j was done by warp 0)
            const int c0 = j + 1, k = j - 1;
            const int w = nb - c0;  // trailing width
            for (int e = wk * 32 + lane; e < w * w; e += nworkers) {
                const int rr = c0 + e / w, cc = c0 + e % w;
                if (cc <= rr) s[rr][cc] = fma(-s[rr][k], s[cc][k], s[rr][cc]);
            }
        }
        __syncthreads();
        if (warp == 0 && j + 1 < nb) {  // lookahead: column j applied to column j+1
            const int r = lane;
            if (r >= j + 1 && r < nb) s[r][j + 1] = fma(-s[r][j], s[j + 1][j], s[r][j + 1]);
        }
    }
    __syncthreads();

    if (tid == 0 && fail != 0 && info != nullptr) atomicCAS(info, 0, (int32_t)(row0 + fail));

    tile_inverse<T>(s, x, tmp, yv);

    for (int e = tid; e < nb * nb; e += NT) {
        const int r = e / nb, c = e - (e / nb) * nb;
        A[(int64_t)r * ld + c] = (c <= r) ? s[r][c] : T(0);
        tinv[r * kTile + c] = x[r][c];
    }
    // The reference's cholesky returns a zero strict upper triangle: clear
    // the part of these rows to the right of the tile.
    for (int e = tid; e < nb * zero_right; e += NT) {
        const int r = e / zero_right, c = e - (e / zero_right) * zero_right;
        A[(int64_t)r * ld + nb + c] = T(0);
    }
}

// grid (tiles, batch): inverse of diagonal tile t of block blockIdx.y.
template <typename T>
__global__ void __launch_bounds__(NT)
k_trtri_tiles(const T* L, int64_t ldl, int64_t strideL, int m, T* X, int64_t ldx, int64_t strideX) {
    __shared__ T s[kTile][kTile + 1];
    __shared__ T x[kTile][kTile + 1];
    __shared__ T tmp[kTile][kTile + 1];
    __shared__ T yv[kTile];
    const int t0 = blockIdx.x * kTile;
    const int nb = min(kTile, m - t0);
    const T* Lb = L + (int64_t)blockIdx.y * strideL + (int64_t)t0 * ldl + t0;
    T* Xb = X + (int64_t)blockIdx.y * strideX + (int64_t)t0 * ldx + t0;
    for (int e = threadIdx.x; e < kTile * kTile; e += NT) {
        const int r = e / kTile, c = e % kTile;
        T v = T(0);
        if (r < nb && c <= r) v = Lb[(int64_t)r * ldl + c];
        else if (r >= nb && r == c) v = T(1);
        s[r][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < kTile) yv[threadIdx.x] = T(1) / s[threadIdx.x][threadIdx.x];
    __syncthreads();
    tile_inverse<T>(s, x, tmp, yv);
    for (int e = threadIdx.x; e < nb * nb; e += NT) {
        const int r = e / nb, c = e - (e / nb) * nb;
        Xb[(int64_t)r * ldx + c] = x[r][c];
    }
}

template <typename T>
GemmProb<T> blank_prob() {
    GemmProb<T> p;
    memset(&p, 0, sizeof(p));
    p.batch = 1;
    p.alpha = T(1);
    p.beta = T(0);
    return p;
}

}  // namespace

template <typename T>
cudaError_t potrf_tile(T* tile, int64_t ld, int nb, int zero_cols_right, T* tinv, int32_t* info,
                       int64_t info_row0, cudaStream_t s) {
    prof_before(s);
    k_potrf_tile<T><<<1, NT, 0, s>>>(tile, ld, nb, zero_cols_right, tinv, info, info_row0);
    prof_after(SGB_KCLASS_POTRF_TILE, s, 2.0 * nb * nb * nb / 3.0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t trtri_tiles_batched(const T* L, int64_t ldl, int64_t strideL, int m, int batch, T* Linv,
                                int64_t ldx, int64_t strideX, cudaStream_t s) {
    if (m <= 0 || batch <= 0) return cudaSuccess;
    dim3 grid((unsigned)ceil_div(m, kTile), (unsigned)batch);
    prof_before(s);
    k_trtri_tiles<T><<<grid, NT, 0, s>>>(L, ldl, strideL, m, Linv, ldx, strideX);
    prof_after(SGB_KCLASS_TRTRI_TILE, s, (double)batch * m * (double)kTile * kTile / 3.0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t factor_column_block(T* diag, int64_t m, int64_t ldd, RowSet<T> r1, RowSet<T> r2, T* scratch,
                                int32_t* info, int64_t info_row0, cudaStream_t s) {
    cudaError_t err;
    for (int64_t c0 = 0; c0 < m; c0 += kTile) {
        const int w = (int)((m - c0) < kTile ? (m - c0) : kTile);
        const int64_t c1 = c0 + w;
        const int64_t right = m - c1;
        err = potrf_tile<T>(diag + c0 * ldd + c0, ldd, w, (int)right, scratch, info, info_row0 + c0, s);
        if (err != cudaSuccess) return err;

        // rows below the tile: P[:, c0:c1] <- P[:, c0:c1] * Ltile^{-T}
        GemmProb<T> pr[3];
        int np = 0;
        auto trsm = [&](T* base, int64_t rows, int64_t ld) {
            if (rows <= 0) return;
            GemmProb<T> p = blank_prob<T>();
            p.M = (int32_t)rows;
            p.N = w;
            p.nterms = 1;
            p.term[0].A = base + c0;
            p.term[0].lda = ld;
            p.term[0].B = scratch;
            p.term[0].ldb = kTile;
            p.term[0].transB = 1;
            p.term[0].K = w;
            p.term[0].kmode = KM_LT_N1;
            p.Cout = base + c0;
            p.ldc = ld;
            pr[np++] = p;
        };
        trsm(diag + c1 * ldd, right, ldd);
        trsm(r1.p, r1.rows, r1.ld);
        trsm(r2.p, r2.rows, r2.ld);
        if (np) {
            err = gemm_simt<T>(pr, np, s);
            if (err != cudaSuccess) return err;
        }
        if (right <= 0) continue;

        // trailing update: P[:, c1:m] -= P[:, c0:c1] * D[c1:m, c0:c1]^T
        np = 0;
        const T* Bpan = diag + c1 * ldd + c0;
        auto upd = [&](T* base, int64_t rows, int64_t ld, int lower) {
            if (rows <= 0) return;
            GemmProb<T> p = blank_prob<T>();
            p.M = (int32_t)rows;
            p.N = (int32_t)right;
            p.nterms = 1;
            p.term[0].A = base + c0;
            p.term[0].lda = ld;
            p.term[0].B = Bpan;
            p.term[0].ldb = ldd;
            p.term[0].transB = 1;
            p.term[0].K = w;
            p.alpha = T(-1);
            p.beta = T(1);
            p.Cin = base + c1;
            p.ldcin = ld;
            p.Cout = base + c1;
            p.ldc = ld;
            p.lower_only = (int8_t)lower;
            pr[np++] = p;
        };
        upd(diag + c1 * ldd, right, ldd, 1);
        upd(r1.p, r1.rows, r1.ld, 0);
        upd(r2.p, r2.rows, r2.ld, 0);
        err = gemm_simt<T>(pr, np, s);
        if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
}

template <typename T>
cudaError_t trtri_batched(const T* L, int64_t ldl, int64_t strideL, int64_t m, int64_t batch, T* Linv,
                          int64_t ldx, int64_t strideX, T* scratch, cudaStream_t s, GemmFn<T> fn, void* fnctx) {
    auto gemm = [&](GemmProb<T>* p) { return fn ? fn(fnctx, p, 1, s) : gemm_simt<T>(p, 1, s); };
    if (m <= 0 || batch <= 0) return cudaSuccess;
    cudaError_t err;
    // Zero the strict upper triangle (and everything else) first; the row
    // sweep writes only the lower tiles.
    if (ldx == m && strideX == m * m) {
        err = cudaMemsetAsync(Linv, 0, (size_t)(batch * m * m) * sizeof(T), s);
    } else {
        err = cudaMemset2DAsync(Linv, (size_t)ldx * sizeof(T), 0, (size_t)m * sizeof(T),
                                (size_t)(m + (batch - 1) * (strideX / ldx)), s);
    }
    if (err != cudaSuccess) return err;
    err = trtri_tiles_batched<T>(L, ldl, strideL, (int)m, (int)batch, Linv, ldx, strideX, s);
    if (err != cudaSuccess) return err;
    for (int64_t r0 = kTile; r0 < m; r0 += kTile) {
        const int rows = (int)((m - r0) < kTile ? (m - r0) : kTile);
        // tmp = L[r0:r0+rows, 0:r0] * Linv[0:r0, 0:r0]
        GemmProb<T> p = blank_prob<T>();
        p.M = rows;
        p.N = (int32_t)r0;
        p.batch = (int32_t)batch;
        p.nterms = 1;
        p.term[0].A = L + r0 * ldl;
        p.term[0].lda = ldl;
        p.term[0].strideA = strideL;
        p.term[0].B = Linv;
        p.term[0].ldb = ldx;
        p.term[0].strideB = strideX;
        p.term[0].K = (int32_t)r0;
        p.term[0].kmode = KM_GE_N0;
        p.Cout = scratch;
        p.ldc = m;
        p.strideC = (int64_t)kTile * m;
        err = gemm(&p);
        if (err != cudaSuccess) return err;
        // Linv[r0:r0+rows, 0:r0] = -Linv[r0:, r0:](tile) * tmp
        GemmProb<T> q = blank_prob<T>();
        q.M = rows;
        q.N = (int32_t)r0;
        q.batch = (int32_t)batch;
        q.nterms = 1;
        q.term[0].A = Linv + r0 * ldx + r0;
        q.term[0].lda = ldx;
        q.term[0].strideA = strideX;
        q.term[0].B = scratch;
        q.term[0].ldb = m;
        q.term[0].strideB = (int64_t)kTile * m;
        q.term[0].K = rows;
        q.term[0].kmode = KM_LT_M1;
        q.alpha = T(-1);
        q.Cout = Linv + r0 * ldx;
        q.ldc = ldx;
        q.strideC = strideX;
        err = gemm(&q);
        if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
}

#define SGB_INST(T)                                                                                      \
    template cudaError_t potrf_tile<T>(T*, int64_t, int, int, T*, int32_t*, int64_t, cudaStream_t);       \
    template cudaError_t trtri_tiles_batched<T>(const T*, int64_t, int64_t, int, int, T*, int64_t,       \
                                                int64_t, cudaStream_t);                                   \
    template cudaError_t factor_column_block<T>(T*, int64_t, int64_t, RowSet<T>, RowSet<T>, T*,          \
                                                int32_t*, int64_t, cudaStream_t);                         \
    template cudaError_t trtri_batched<T>(const T*, int64_t, int64_t, int64_t, int64_t, T*, int64_t,     \
                                          int64_t, T*, cudaStream_t, GemmFn<T>, void*);
SGB_INST(double)
SGB_INST(float)

}  // namespace sgb
