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
// * trtri_batched: L^{-1} of many blocks at once (recursive doubling over
//   32-row tiles: a handful of grouped, batched products per level).
#include <math.h>
#include <string.h>

#include "sgb_internal.cuh"
#include "sgb_tile.cuh"

namespace sgb {

namespace {

constexpr int NT = kTileThreads;

// Diagonal tile: Cholesky + inverse (sgb_tile.cuh), pivot reported to info.
template <typename T>
__global__ void __launch_bounds__(NT)
k_potrf_tile(T* A, int64_t ld, int nb, int zero_right, T* tinv, int32_t* info, int64_t row0) {
    __shared__ Smem<T> S;
    factor_tile<T>(S, A, ld, nb, zero_right, tinv, info, row0);
}

// grid (tiles, batch): inverse of diagonal tile t of block blockIdx.y.
template <typename T>
__global__ void __launch_bounds__(NT)
k_trtri_tiles(const T* L, int64_t ldl, int64_t strideL, int m, T* X, int64_t ldx, int64_t strideX) {
    __shared__ Smem<T> S;
    const int t0 = blockIdx.x * kTile;
    const int nb = min(kTile, m - t0);
    const T* Lb = L + (int64_t)blockIdx.y * strideL + (int64_t)t0 * ldl + t0;
    T* Xb = X + (int64_t)blockIdx.y * strideX + (int64_t)t0 * ldx + t0;
    for (int e = threadIdx.x; e < kTile * kTile; e += NT) {
        const int r = e / kTile, c = e % kTile;
        T v = T(0);
        if (r < nb && c <= r) v = Lb[(int64_t)r * ldl + c];
        else if (r >= nb && r == c) v = T(1);
        S.s[r][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < kTile) S.yv[threadIdx.x] = T(1) / S.s[threadIdx.x][threadIdx.x];
    __syncthreads();
    tile_inverse_dev<T>(S);
    for (int e = threadIdx.x; e < nb * nb; e += NT) {
        const int r = e / nb, c = e - (e / nb) * nb;
        Xb[(int64_t)r * ldx + c] = S.x[r][c];
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
    prof_before(s, SGB_KCLASS_POTRF_TILE);
    k_potrf_tile<T><<<1, NT, 0, s>>>(tile, ld, nb, zero_cols_right, tinv, info, info_row0);
    prof_after(SGB_KCLASS_POTRF_TILE, s, 2.0 * nb * nb * nb / 3.0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t trtri_tiles_batched(const T* L, int64_t ldl, int64_t strideL, int m, int batch, T* Linv,
                                int64_t ldx, int64_t strideX, cudaStream_t s) {
    if (m <= 0 || batch <= 0) return cudaSuccess;
    dim3 grid((unsigned)ceil_div(m, kTile), (unsigned)batch);
    prof_before(s, SGB_KCLASS_TRTRI_TILE);
    k_trtri_tiles<T><<<grid, NT, 0, s>>>(L, ldl, strideL, m, Linv, ldx, strideX);
    prof_after(SGB_KCLASS_TRTRI_TILE, s, (double)batch * m * (double)kTile * kTile / 3.0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t factor_column_block(T* diag, int64_t m, int64_t ldd, RowSet<T> r1, RowSet<T> r2, T* scratch,
                                int32_t* info, int64_t info_row0, cudaStream_t s, RowSet<T> r3) {
    cudaError_t err;
    for (int64_t c0 = 0; c0 < m; c0 += kTile) {
        const int w = (int)((m - c0) < kTile ? (m - c0) : kTile);
        const int64_t c1 = c0 + w;
        const int64_t right = m - c1;
        err = potrf_tile<T>(diag + c0 * ldd + c0, ldd, w, (int)right, scratch, info, info_row0 + c0, s);
        if (err != cudaSuccess) return err;

        // rows below the tile: P[:, c0:c1] <- P[:, c0:c1] * Ltile^{-T}
        GemmProb<T> pr[4];
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
        trsm(r3.p, r3.rows, r3.ld);
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
        upd(r3.p, r3.rows, r3.ld, 0);
        err = gemm_simt<T>(pr, np, s);
        if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
}

template <typename T>
cudaError_t trtri_batched(const T* L, int64_t ldl, int64_t strideL, int64_t m, int64_t batch, T* Linv,
                          int64_t ldx, int64_t strideX, T* scratch, cudaStream_t s, GemmFn<T> fn, void* fnctx) {
    auto gemm = [&](GemmProb<T>* p, int np) { return fn ? fn(fnctx, p, np, s) : gemm_simt<T>(p, np, s); };
    if (m <= 0 || batch <= 0) return cudaSuccess;
    cudaError_t err;
    // Zero everything first: the recursion writes only the lower blocks.
    if (ldx == m && strideX == m * m) {
        err = cudaMemsetAsync(Linv, 0, (size_t)(batch * m * m) * sizeof(T), s);
    } else {
        err = cudaMemset2DAsync(Linv, (size_t)ldx * sizeof(T), 0, (size_t)m * sizeof(T),
                                (size_t)(m + (batch - 1) * (strideX / ldx)), s);
    }
    if (err != cudaSuccess) return err;
    err = trtri_tiles_batched<T>(L, ldl, strideL, (int)m, (int)batch, Linv, ldx, strideX, s);
    if (err != cudaSuccess) return err;
    // Recursive doubling: at level h, every pair of h-blocks along the
    // diagonal, [L11 0; L21 L22], gets X21 = -X22 (L21 X11) from the inverses
    // X11, X22 of the level below.  Pairs of a level are independent and go
    // four to a grouped launch; every problem is batched over the blocks.
    // Scratch per block: the products L21 X11 of one level (<= m*m/2 + h*h).
    const int64_t sstride = m * m;
    for (int64_t h = kTile; h < m; h *= 2) {
        int64_t q = 0;
        while ((2 * q + 1) * h < m) {
            GemmProb<T> pr[4], pq[4];
            int np = 0;
            for (; np < 4 && (2 * q + 1) * h < m; ++np, ++q) {
                const int64_t r1 = (2 * q + 1) * h, c0 = 2 * q * h;
                const int64_t rows2 = (m - r1) < h ? (m - r1) : h;
                T* tq = scratch + q * h * h;
                GemmProb<T> p = blank_prob<T>();  // T = L21 X11
                p.M = (int32_t)rows2;
                p.N = (int32_t)h;
                p.batch = (int32_t)batch;
                p.nterms = 1;
                p.term[0].A = L + r1 * ldl + c0;
                p.term[0].lda = ldl;
                p.term[0].strideA = strideL;
                p.term[0].B = Linv + c0 * ldx + c0;
                p.term[0].ldb = ldx;
                p.term[0].strideB = strideX;
                p.term[0].K = (int32_t)h;
                p.term[0].kmode = KM_GE_N0;
                p.Cout = tq;
                p.ldc = h;
                p.strideC = sstride;
                pr[np] = p;
                GemmProb<T> w = blank_prob<T>();  // X21 = -X22 T
                w.M = (int32_t)rows2;
                w.N = (int32_t)h;
                w.batch = (int32_t)batch;
                w.nterms = 1;
                w.term[0].A = Linv + r1 * ldx + r1;
                w.term[0].lda = ldx;
                w.term[0].strideA = strideX;
                w.term[0].B = tq;
                w.term[0].ldb = h;
                w.term[0].strideB = sstride;
                w.term[0].K = (int32_t)rows2;
                w.term[0].kmode = KM_LT_M1;
                w.alpha = T(-1);
                w.Cout = Linv + r1 * ldx + c0;
                w.ldc = ldx;
                w.strideC = strideX;
                pq[np] = w;
            }
            err = gemm(pr, np);
            if (err != cudaSuccess) return err;
            err = gemm(pq, np);
            if (err != cudaSuccess) return err;
        }
    }
    return cudaSuccess;
}

#define SGB_INST(T)                                                                                      \
    template cudaError_t potrf_tile<T>(T*, int64_t, int, int, T*, int32_t*, int64_t, cudaStream_t);       \
    template cudaError_t trtri_tiles_batched<T>(const T*, int64_t, int64_t, int, int, T*, int64_t,       \
                                                int64_t, cudaStream_t);                                   \
    template cudaError_t factor_column_block<T>(T*, int64_t, int64_t, RowSet<T>, RowSet<T>, T*,          \
                                                int32_t*, int64_t, cudaStream_t, RowSet<T>);              \
    template cudaError_t trtri_batched<T>(const T*, int64_t, int64_t, int64_t, int64_t, T*, int64_t,     \
                                          int64_t, T*, cudaStream_t, GemmFn<T>, void*);
SGB_INST(double)
SGB_INST(float)

}  // namespace sgb
