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
//   C(p)  CTAs 1-4 first update the next diagonal tile (p+1, p+1), eight
//         rows each, and count themselves on a flag; CTA 0 waits for the
//         flag and factors that tile at once (lookahead) while CTAs 1..
//         apply the rank-32 update to the rest of the trailing panel.  The
//         barrier after A(p+1) also closes C(p), which B(p+1) needs.
//
// Grid barriers are a counter + generation pair in global memory with a
// bounded spin: a barrier that does not complete within the limit sets the
// status word to SGB_ERR_TIMEOUT and every CTA leaves the kernel (the
// cooperative launch guarantees that all CTAs are resident, so a complete
// barrier never waits on an unscheduled CTA).  Data produced by other CTAs
// is read with ld.global.cg (L2), never from a possibly stale L1 line.
#include <math.h>

#include "sgb_internal.cuh"
#include "sgb_tile.cuh"

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
    unsigned* bar;    // [0] arrivals, [1] generation, [2] diagonal-tile pieces; zero at launch
    int32_t* status;  // SGB_ERR_TIMEOUT on a stuck barrier
};

template <typename T>
__device__ __forceinline__ T ldcg(const T* p) {
    return __ldcg(p);
}

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
__global__ void __launch_bounds__(NT, 1) k_factor_panel(const __grid_constant__ PanelArgs<T> a) {
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
            // (strip * tinv^T)[ty][tx] = sum_{k <= tx} strip[ty][k] tinv[tx][k], four accumulators
            const int kend = (tx < w - 1 ? tx : w - 1) + 1;
            T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
            int k = 0;
            for (; k + 3 < kend; k += 4) {
                a0 = fma(S.tmp[ty][k], S.x[tx][k], a0);
                a1 = fma(S.tmp[ty][k + 1], S.x[tx][k + 1], a1);
                a2 = fma(S.tmp[ty][k + 2], S.x[tx][k + 2], a2);
                a3 = fma(S.tmp[ty][k + 3], S.x[tx][k + 3], a3);
            }
            for (; k < kend; ++k) a0 = fma(S.tmp[ty][k], S.x[tx][k], a0);
            if (rp != nullptr && tx < w) rp[tx] = (a0 + a1) + (a2 + a3);
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
        // The next diagonal tile (p+1, p+1) is on the critical path: CTAs
        // 1-4 update 8 of its rows each (lower part) and publish them on a
        // counter; CTA 0 waits for the four pieces and factors the tile
        // while the other CTAs run the rest of the trailing update.
        if (blockIdx.x == 0) {
            if (tid == 0) {
                const unsigned target = 4u * (unsigned)(p + 1);
                long long spins = 0;
                int ok = 1;
                while (atomicAdd(&a.bar[2], 0u) < target) {
                    if (++spins > kBarrierSpin) {
                        ok = 0;
                        atomicExch(a.status, SGB_ERR_TIMEOUT);
                        break;
                    }
                    __nanosleep(32);
                }
                __threadfence();
                S.flag = ok;
            }
            __syncthreads();
            if (!S.flag) return;
            const int w2 = (int)((m - c1) < kTile ? (m - c1) : kTile);
            factor_tile<T>(S, a.diag + c1 * a.ldd + c1, a.ldd, w2, (int)(m - c1 - w2), a.tinv, a.info,
                           a.row0 + c1);
        } else {
            if (blockIdx.x <= 4) {
                const int piece = (int)blockIdx.x - 1;
                const int64_t rows_d = (m - c1) < kTile ? (m - c1) : kTile;
                for (int e = tid; e < kTile * kTile; e += NT) {
                    const int r = e / kTile, k = e % kTile;
                    S.tmp[r][k] = (r < rows_d && k < w) ? ldcg(Bpan + (int64_t)r * a.ldd + k) : T(0);
                }
                __syncthreads();
                const int r = piece * 8 + ty, c = tx;
                if (r < rows_d && c <= r) {
                    T acc = T(0);
                    for (int k = 0; k < w; ++k) acc = fma(S.tmp[r][k], S.tmp[c][k], acc);
                    T* cp = a.diag + (c1 + r) * a.ldd + c1 + c;
                    *cp = ldcg(cp) - acc;
                }
                __threadfence();
                __syncthreads();
                if (tid == 0) atomicAdd(&a.bar[2], 1u);
            }
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
        int per = occ < 1 ? occ : 1;  // one CTA per SM: cheaper barriers, full FP64 pipe per CTA
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
    e = cudaMemsetAsync(bar, 0, 3 * sizeof(unsigned), s);
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
