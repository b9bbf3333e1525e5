// Persistent, cooperative factorization of one BTA column block
// [D_i; Lo_i; Ar_i] (the tall panel of pobtaf, src/serinv/algs/pobtaf.py:
// 117-139) in a single launch.
//
// The launch-based sweep (factor_column_block) issues three kernels per
// 32-wide tile column: the diagonal-tile Cholesky, the strip TRSM and the
// rank-32 trailing update.  Here one cooperative grid runs all tile columns:
//
//   A(p)  CTA 0 factors diagonal tile p (and forms its inverse);
//   --- grid barrier ---
//   B(p)  all CTAs: rows below the tile <- rows * tile^{-T} (8-row chunks);
//   --- grid barrier ---
//   C(p)  CTA 0 updates only the next diagonal tile (p+1, p+1) and moves on
//         to A(p+1) at once (lookahead); CTAs 1.. apply the rank-32 update
//         to the rest of the trailing panel.  The barrier after A(p+1) also
//         closes C(p), which B(p+1) needs.
//
// Grid barriers are a counter + generation pair in global memory with a
// bounded spin: a barrier that does not complete within the limit sets the
// status word to SGB_ERR_TIMEOUT and every CTA leaves the kernel (the
// cooperative launch guarantees that all CTAs are resident, so a complete
// barrier never waits on an unscheduled CTA).  Data produced by other CTAs
// is read with ld.global.cg (L2), never from a possibly stale L1 line.
#include <math.h>

#include "sgb_internal.cuh"

namespace sgb {

namespace {

constexpr int NT = 256;
constexpr long long kBarrierSpin = 1ll << 22;

template <typename T>
struct PanelArgs {
    T* diag;
    int64_t m, ldd;
    T* r1;
    int64_t r1rows, r1ld;
    T* r2;
    int64_t r2rows, r2ld;
    T* tinv;  // 32 x 32 global scratch
    int32_t* info;
    int64_t row0;
    unsigned* bar;    // [0] arrivals, [1] generation; zero at launch
    int32_t* status;  // SGB_ERR_TIMEOUT on a stuck barrier
};

template <typename T>
__device__ __forceinline__ T ldcg(const T* p) {
    return __ldcg(p);
}

template <typename T>
__device__ __forceinline__ T rsq(T x);
template <>
__device__ __forceinline__ double rsq<double>(double x) { return rsqrt(x); }
template <>
__device__ __forceinline__ float rsq<float>(float x) { return rsqrtf(x); }

// Grid barrier; returns false (on every thread of the CTA) if it timed out.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, unsigned& epoch, int32_t* status,
                                             int* sflag) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned target = epoch + 1;
        int ok = 1;
        if (atomicAdd(&bar[0], 1u) == nblocks - 1) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicExch(&bar[1], target);
        } else {
            long long spins = 0;
            while ((int)(atomicAdd(&bar[1], 0u) - target) < 0) {
                if (++spins > kBarrierSpin) {
                    ok = 0;
                    atomicExch(status, SGB_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        epoch = target;
        *sflag = ok && (atomicAdd((unsigned*)status, 0u) == 0u);
    }
    __syncthreads();
    return *sflag != 0;
}

template <typename T>
struct Smem {
    T s[kTile][kTile + 1];
    T x[kTile][kTile + 1];
    T tmp[kTile][kTile + 1];
    T yv[kTile];
    int fail;
    int flag;
};

// Recursive-doubling inverse of the (identity padded) lower tile s into x.
template <typename T>
__device__ void tile_inverse_dev(Smem<T>& S) {
    const int tid = threadIdx.x;
    for (int e = tid; e < kTile * kTile; e += NT) S.x[e / kTile][e % kTile] = T(0);
    __syncthreads();
    if (tid < 32) {
        const int blk = tid >> 3, jj = tid & 7, b0 = blk * 8, j = b0 + jj;
        for (int r = j; r < b0 + 8; ++r) {
            T sum = (r == j) ? T(1) : T(0);
            for (int k = j; k < r; ++k) sum = fma(-S.s[r][k], S.x[k][j], sum);
            S.x[r][j] = sum * S.yv[r];
        }
    }
    __syncthreads();
    for (int h = 8; h < kTile; h *= 2) {
        const int nblk = kTile / (2 * h);
        for (int e = tid; e < nblk * h * h; e += NT) {
            const int bi = e / (h * h), rem = e % (h * h), r = rem / h, c = rem % h, o = bi * 2 * h;
            T sum = T(0);
            for (int k = c; k < h; ++k) sum = fma(S.s[o + h + r][o + k], S.x[o + k][o + c], sum);
            S.tmp[o + h + r][o + c] = sum;
        }
        __syncthreads();
        for (int e = tid; e < nblk * h * h; e += NT) {
            const int bi = e / (h * h), rem = e % (h * h), r = rem / h, c = rem % h, o = bi * 2 * h;
            T sum = T(0);
            for (int k = 0; k <= r; ++k) sum = fma(S.x[o + h + r][o + h + k], S.tmp[o + h + k][o + c], sum);
            S.x[o + h + r][o + c] = -sum;
        }
        __syncthreads();
    }
}

// A(p): Cholesky + inverse of the diagonal tile at `tile` (nb <= 32), by one CTA.
template <typename T>
__device__ void factor_tile(Smem<T>& S, T* tile, int64_t ld, int nb, int zero_right, T* tinv, int32_t* info,
                            int64_t row0) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int e = tid; e < kTile * kTile; e += NT) {
        const int r = e / kTile, c = e % kTile;
        T v = T(0);
        if (r < nb && c <= r) v = ldcg(tile + (int64_t)r * ld + c);
        else if (r >= nb && r == c) v = T(1);
        S.s[r][c] = v;
    }
    if (tid == 0) S.fail = 0;
    if (tid < kTile) S.yv[tid] = T(1);
    __syncthreads();
    const int wk = warp == 0 || warp == 4 ? -1 : (warp < 4 ? warp - 1 : warp - 2);
    for (int j = 0; j < nb; ++j) {
        if (warp == 0) {
            const T d = S.s[j][j];
            const bool bad = !(d > T(0)) || !isfinite((double)d);
            const T y = bad ? T(NAN) : rsq<T>(d);
            if (lane > j && lane < nb) S.s[lane][j] *= y;
            if (lane == j) {
                S.s[j][j] = d * y;
                S.yv[j] = y;
                if (bad && S.fail == 0) S.fail = j + 1;
            }
        } else if (wk >= 0 && j >= 1) {
            const int c0 = j + 1, k = j - 1, w = nb - c0;
            for (int e = wk * 32 + lane; e < w * w; e += 6 * 32) {
                const int rr = c0 + e / w, cc = c0 + e % w;
                if (cc <= rr) S.s[rr][cc] = fma(-S.s[rr][k], S.s[cc][k], S.s[rr][cc]);
            }
        }
        __syncthreads();
        if (warp == 0 && j + 1 < nb && lane >= j + 1 && lane < nb)
            S.s[lane][j + 1] = fma(-S.s[lane][j], S.s[j + 1][j], S.s[lane][j + 1]);
    }
    __syncthreads();
    if (tid == 0 && S.fail != 0 && info != nullptr) atomicCAS(info, 0, (int32_t)(row0 + S.fail));
    tile_inverse_dev<T>(S);
    for (int e = tid; e < nb * nb; e += NT) {
        const int r = e / nb, c = e % nb;
        tile[(int64_t)r * ld + c] = (c <= r) ? S.s[r][c] : T(0);
        tinv[r * kTile + c] = S.x[r][c];
    }
    for (int e = tid; e < nb * zero_right; e += NT) {
        const int r = e / zero_right, c = e % zero_right;
        tile[(int64_t)r * ld + nb + c] = T(0);
    }
}

// Row r of the unified row space [D rows c1..m) ++ r1 rows ++ r2 rows.
template <typename T>
__device__ __forceinline__ T* row_ptr(const PanelArgs<T>& a, int64_t c1, int64_t r) {
    const int64_t nd = a.m - c1;
    if (r < nd) return a.diag + (c1 + r) * a.ldd;
    r -= nd;
    if (r < a.r1rows) return a.r1 + r * a.r1ld;
    return a.r2 + (r - a.r1rows) * a.r2ld;
}

template <typename T>
__global__ void __launch_bounds__(NT) k_factor_panel(const __grid_constant__ PanelArgs<T> a) {
    __shared__ Smem<T> S;
    const int tid = threadIdx.x;
    const unsigned G = gridDim.x;
    unsigned epoch = 0;
    const int64_t m = a.m;
    const int64_t nt = (m + kTile - 1) / kTile;
    const int tx = tid & 31, ty = tid >> 5;

    // A(0)
    if (blockIdx.x == 0)
        factor_tile<T>(S, a.diag, a.ldd, (int)(m < kTile ? m : kTile), (int)(m > kTile ? m - kTile : 0), a.tinv,
                       a.info, a.row0);
    if (!grid_barrier(a.bar, G, epoch, a.status, &S.flag)) return;

    for (int64_t p = 0; p < nt; ++p) {
        const int64_t c0 = p * kTile;
        const int w = (int)((m - c0) < kTile ? (m - c0) : kTile);
        const int64_t c1 = c0 + w;
        const int64_t nrows = (m - c1) + a.r1rows + a.r2rows;

        // B(p): strip TRSM, 8-row chunks; tinv^T applied from shared memory
        for (int e = tid; e < kTile * kTile; e += NT) S.x[e / kTile][e % kTile] = ldcg(a.tinv + e);
        __syncthreads();
        for (int64_t ch = blockIdx.x; ch * 8 < nrows; ch += G) {
            const int64_t r = ch * 8 + ty;
            T* rp = r < nrows ? row_ptr(a, c1, r) + c0 : nullptr;
            S.tmp[ty][tx] = (rp != nullptr && tx < w) ? ldcg(rp + tx) : T(0);
            __syncthreads();
            T acc = T(0);
            for (int k = 0; k <= tx && k < w; ++k) acc = fma(S.tmp[ty][k], S.x[tx][k], acc);
            if (rp != nullptr && tx < w) rp[tx] = acc;
            __syncthreads();
        }
        if (!grid_barrier(a.bar, G, epoch, a.status, &S.flag)) return;
        if (c1 >= m) break;

        // C(p): rank-w update of the trailing panel
        const int64_t ntd = (m - c1 + kTile - 1) / kTile;
        const int64_t n1 = (a.r1rows + kTile - 1) / kTile, n2 = (a.r2rows + kTile - 1) / kTile;
        const int64_t tiles_d = ntd * (ntd + 1) / 2;
        const int64_t total = tiles_d + (n1 + n2) * ntd;
        const T* Bpan = a.diag + c1 * a.ldd + c0;
        auto do_tile = [&](int64_t t) {
            T* Cbase;
            const T* Abase;
            int64_t ldc, rows, cj;
            if (t < tiles_d) {  // lower tiles of the trailing D, row-major over the triangle
                int64_t ti = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
                while (ti * (ti + 1) / 2 > t) --ti;
                while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
                cj = t - ti * (ti + 1) / 2;
                Cbase = a.diag + (c1 + ti * kTile) * a.ldd + c1;
                Abase = a.diag + (c1 + ti * kTile) * a.ldd + c0;
                ldc = a.ldd;
                rows = (m - c1) - ti * kTile;
            } else if (t < tiles_d + n1 * ntd) {
                const int64_t u = t - tiles_d, ti = u / ntd;
                cj = u % ntd;
                Cbase = a.r1 + ti * kTile * a.r1ld + c1;
                Abase = a.r1 + ti * kTile * a.r1ld + c0;
                ldc = a.r1ld;
                rows = a.r1rows - ti * kTile;
            } else {
                const int64_t u = t - tiles_d - n1 * ntd, ti = u / ntd;
                cj = u % ntd;
                Cbase = a.r2 + ti * kTile * a.r2ld + c1;
                Abase = a.r2 + ti * kTile * a.r2ld + c0;
                ldc = a.r2ld;
                rows = a.r2rows - ti * kTile;
            }
            if (rows > kTile) rows = kTile;
            int64_t cols = (m - c1) - cj * kTile;
            if (cols > kTile) cols = kTile;
            // stage A (rows x w) and B (cols x w) in shared memory
            for (int e = tid; e < kTile * kTile; e += NT) {
                const int r = e / kTile, k = e % kTile;
                S.s[r][k] = (r < rows && k < w) ? ldcg(Abase + (int64_t)r * ldc + k) : T(0);
                S.tmp[r][k] = (r < cols && k < w) ? ldcg(Bpan + (cj * kTile + r) * a.ldd + k) : T(0);
            }
            __syncthreads();
            const int cx = tid & 15, cy = tid >> 4;
            T acc[2][2] = {{T(0), T(0)}, {T(0), T(0)}};
            for (int k = 0; k < w; ++k) {
                const T a0 = S.s[cy][k], a1 = S.s[cy + 16][k];
                const T b0 = S.tmp[cx][k], b1 = S.tmp[cx + 16][k];
                acc[0][0] = fma(a0, b0, acc[0][0]);
                acc[0][1] = fma(a0, b1, acc[0][1]);
                acc[1][0] = fma(a1, b0, acc[1][0]);
                acc[1][1] = fma(a1, b1, acc[1][1]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const int r = cy + 16 * i, c = cx + 16 * j;
                    if (r < rows && c < cols) {
                        T* cp = Cbase + (int64_t)r * ldc + cj * kTile + c;
                        *cp = ldcg(cp) - acc[i][j];
                    }
                }
            __syncthreads();
        };
        if (blockIdx.x == 0) {
            do_tile(0);  // the next diagonal tile, then its factorization right away
            const int64_t c2 = c1;
            const int w2 = (int)((m - c2) < kTile ? (m - c2) : kTile);
            factor_tile<T>(S, a.diag + c2 * a.ldd + c2, a.ldd, w2, (int)(m - c2 - w2), a.tinv, a.info,
                           a.row0 + c2);
        } else {
            for (int64_t t = 1 + (blockIdx.x - 1); t < total; t += (G > 1 ? G - 1 : 1)) do_tile(t);
        }
        if (!grid_barrier(a.bar, G, epoch, a.status, &S.flag)) return;
    }
}

int g_panel_grid[64] = {};

}  // namespace

template <typename T>
cudaError_t factor_panel_persistent(T* diag, int64_t m, int64_t ldd, RowSet<T> r1, RowSet<T> r2, T* tinv,
                                    unsigned* bar, int32_t* status, int32_t* info, int64_t info_row0,
                                    cudaStream_t s) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (g_panel_grid[dev] == 0) {
        int sms = 0, occ = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_factor_panel<double>, NT, 0);
        if (e != cudaSuccess) return e;
        int per = occ < 2 ? occ : 2;
        if (per < 1) return cudaErrorLaunchOutOfResources;
        g_panel_grid[dev] = sms * per;
    }
    const int G = g_panel_grid[dev];
    PanelArgs<T> a;
    a.diag = diag;
    a.m = m;
    a.ldd = ldd;
    a.r1 = r1.p;
    a.r1rows = r1.p ? r1.rows : 0;
    a.r1ld = r1.ld;
    a.r2 = r2.p;
    a.r2rows = r2.p ? r2.rows : 0;
    a.r2ld = r2.ld;
    a.tinv = tinv;
    a.info = info;
    a.row0 = info_row0;
    a.bar = bar;
    a.status = status;
    e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    void* args[] = {(void*)&a};
    prof_before(s);
    e = cudaLaunchCooperativeKernel((const void*)k_factor_panel<T>, dim3(G), dim3(NT), args, 0, s);
    prof_after(SGB_KCLASS_PANEL, s, 0.0);
    return e;
}

template cudaError_t factor_panel_persistent<double>(double*, int64_t, int64_t, RowSet<double>, RowSet<double>,
                                                     double*, unsigned*, int32_t*, int32_t*, int64_t,
                                                     cudaStream_t);
template cudaError_t factor_panel_persistent<float>(float*, int64_t, int64_t, RowSet<float>, RowSet<float>,
                                                    float*, unsigned*, int32_t*, int32_t*, int64_t, cudaStream_t);

}  // namespace sgb
