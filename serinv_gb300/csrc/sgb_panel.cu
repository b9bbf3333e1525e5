// Persistent, cooperative factorization of one BTA column block
// [D_i; Lo_i; Ar_i] (the tall panel of pobtaf, src/serinv/algs/pobtaf.py:
// 117-139) in a single launch.
//
// The launch-based sweep (factor_column_block) issues three kernels per
// 32-wide tile column: the diagonal-tile Cholesky, the strip TRSM and the
// rank-32 trailing update.  Here one cooperative grid runs all tile columns,
// with the chain from one diagonal tile to the next kept as short as the
// FP64 pipe allows.  Roles (G CTAs, one per SM):
//
//   CTA 0        factorizer: diagonal tile p as L = M D^{1/2} (the pivot
//                pipeline of factor_tile_m), publishes M and the pivots d
//                (counter F), then waits for the helpers (counter H2)
//                before tile p+1;
//   CTAs 1..kNH  helpers: once M_p is out, the rows of tile-row p+1 in
//                column block p by unit-triangular substitution
//                (Y M^T = B, X = Y D^{-1/2}; counter H1), then their rows
//                of the update of tile (p+1, p+1) (counter H2); after
//                barrier B they apply column block p to their rows of
//                tile-row p+2 (tiles (p+2, p+1) and (p+2, p+2)), so
//                nothing the next step needs waits for the bulk update;
//   CTA kNH+1    inverter: from M_p, d_p the tile's L (into the matrix)
//                and L^{-1} (for the bulk TRSM; counter I);
//   CTAs kNH+2.. workers: the other rows below tile p times L_pp^{-T}
//                (after I), barrier B (with the helpers), the rank-32
//                update of the rest of the trailing panel, barrier C
//                (workers only).
//
// M/d and L^{-1} alternate between two buffers by the parity of p; the
// factorizer waits for the inverter before overwriting a buffer.  Every
// wait is a bounded poll of a word in global memory: one that does not
// complete within the limit sets the status word to SGB_ERR_TIMEOUT and the
// CTA leaves (the cooperative launch guarantees that all CTAs are
// resident, so no wait depends on an unscheduled CTA).  Data produced by
// other CTAs is read with ld.global.cg (L2), never from a possibly stale
// L1 line.
#include <math.h>

#include "sgb_internal.cuh"
#include "sgb_tile.cuh"

namespace sgb {

namespace {

constexpr int NT = 256;
constexpr long long kBarrierSpin = 1ll << 22;
constexpr int kNH = 8;                 // helper CTAs of the next diagonal tile
constexpr int kHelpRows = kTile / kNH;  // rows of a tile-row per helper
constexpr int kInv = kNH + 1;           // the inverter CTA
constexpr int kW0 = kNH + 2;            // first worker CTA

template <typename T>
struct PanelArgs {
    T* diag;
    int64_t m, ldd;
    T* r1;
    int64_t r1rows, r1ld;
    T* r2;
    int64_t r2rows, r2ld;
    T* scratch;  // [2][32][32] L^{-1}, [2][32][32] M, [2][32] d
    int32_t* info;
    int64_t row0;
    unsigned* bar;    // [0] F, [1] I, [2] H1, [3] H2, [4..5] barrier B, [6..7] barrier C; zero at launch
    int32_t* status;  // SGB_ERR_TIMEOUT on a stuck wait
};

template <typename T>
__device__ __forceinline__ T ldcg(const T* p) {
    return __ldcg(p);
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ bool status_bad(const int32_t* status) {
    return ld_acquire((const unsigned*)status) != 0u;
}

// Barrier over `nblocks` CTAs on the counter/generation pair cg[0], cg[1];
// returns false (on every thread of the CTA) if it timed out.
__device__ __forceinline__ bool group_barrier(unsigned* cg, unsigned nblocks, unsigned& epoch, int32_t* status,
                                              int* sflag) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned target = epoch + 1;
        int ok = 1;
        if (atomicAdd(&cg[0], 1u) == nblocks - 1) {
            atomicExch(&cg[0], 0u);
            __threadfence();
            atomicExch(&cg[1], target);
        } else {
            long long spins = 0;
            while ((int)(ld_acquire(&cg[1]) - target) < 0) {
                if (++spins > kBarrierSpin || status_bad(status)) {
                    ok = 0;
                    atomicExch(status, SGB_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        epoch = target;
        *sflag = ok && !status_bad(status);
    }
    __syncthreads();
    return *sflag != 0;
}

// Wait until *ctr >= target; false (on every thread) on a timeout or an
// error raised elsewhere.
__device__ __forceinline__ bool wait_count(const unsigned* ctr, unsigned target, int32_t* status, int* sflag) {
    if (threadIdx.x == 0) {
        long long spins = 0;
        int ok = 1;
        while (ld_acquire(ctr) < target) {
            if (++spins > kBarrierSpin || status_bad(status)) {
                ok = 0;
                atomicExch(status, SGB_ERR_TIMEOUT);
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
        *sflag = ok;
    }
    __syncthreads();
    return *sflag != 0;
}

// Publish: make this CTA's global writes visible, then count on ctr.
__device__ __forceinline__ void signal(unsigned* ctr) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(ctr, 1u);
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

// rows[ty] (ty < 8) <- rows * tinv^T over the w columns from c0, with tinv
// in S.x; S.tmp is scratch.  Four accumulators per output.
template <typename T>
__device__ __forceinline__ void trsm_rows(Smem<T>& S, T* rp, int w) {
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    S.tmp[ty][tx] = (rp != nullptr && tx < w) ? ldcg(rp + tx) : T(0);
    __syncthreads();
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

// dst[32 x 32] <- rows x cols block of a row-major source (zero padded).
template <typename T>
__device__ __forceinline__ void load_block(T (*dst)[kTile + 1], const T* src, int64_t ld, int rows, int cols) {
    for (int e = threadIdx.x; e < kTile * kTile; e += NT) {
        const int r = e / kTile, c = e % kTile;
        dst[r][c] = (r < rows && c < cols) ? ldcg(src + (int64_t)r * ld + c) : T(0);
    }
}

// out = sum_k a[k] b[k] over k < w, four accumulators.
template <typename T>
__device__ __forceinline__ T dot32(const T* a, const T* b, int w) {
    T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
    int k = 0;
    for (; k + 3 < w; k += 4) {
        a0 = fma(a[k], b[k], a0);
        a1 = fma(a[k + 1], b[k + 1], a1);
        a2 = fma(a[k + 2], b[k + 2], a2);
        a3 = fma(a[k + 3], b[k + 3], a3);
    }
    for (; k < w; ++k) a0 = fma(a[k], b[k], a0);
    return (a0 + a1) + (a2 + a3);
}

template <typename T>
__global__ void __launch_bounds__(NT, 1) k_factor_panel(const __grid_constant__ PanelArgs<T> a) {
    __shared__ Smem<T> S;
    const int tid = threadIdx.x;
    const unsigned G = gridDim.x;
    const unsigned cta = blockIdx.x;
    const int64_t m = a.m;
    const int64_t nt = (m + kTile - 1) / kTile;
    const int tx = tid & 31, ty = tid >> 5;
    unsigned* F = a.bar + 0;
    unsigned* I = a.bar + 1;
    unsigned* H1 = a.bar + 2;
    unsigned* H2 = a.bar + 3;
    unsigned* barB = a.bar + 4;
    unsigned* barC = a.bar + 6;
    T* tinvg = a.scratch;                    // [2][32*32]
    T* Mg = a.scratch + 2 * kTile * kTile;   // [2][32*32]
    T* dg = a.scratch + 4 * kTile * kTile;   // [2][32]
    auto tile_w = [&](int64_t p) -> int { return (int)((m - p * kTile) < kTile ? (m - p * kTile) : kTile); };

    if (cta == 0) {
        // ---------------- factorizer
        for (int64_t p = 0; p < nt; ++p) {
            const int64_t c0 = p * kTile;
            const int w = tile_w(p);
            if (p >= 1 && !wait_count(H2, (unsigned)(kNH * p), a.status, &S.flag)) return;
            if (p >= 2 && !wait_count(I, (unsigned)(p - 1), a.status, &S.flag)) return;
            factor_tile_m<T>(S, a.diag + c0 * a.ldd + c0, a.ldd, w, a.info, a.row0 + c0);
            T* Mo = Mg + (p & 1) * kTile * kTile;
            T* dout = dg + (p & 1) * kTile;
            for (int e = tid; e < kTile * kTile; e += NT) Mo[e] = S.x[e / kTile][e % kTile];
            if (tid < kTile) dout[tid] = S.yv[tid];
            signal(F);
        }
        return;
    }
    if (cta == (unsigned)kInv) {
        // ---------------- inverter
        for (int64_t p = 0; p < nt; ++p) {
            const int64_t c0 = p * kTile;
            const int w = tile_w(p);
            if (!wait_count(F, (unsigned)(p + 1), a.status, &S.flag)) return;
            load_block<T>(S.x, Mg + (p & 1) * kTile * kTile, kTile, kTile, kTile);
            if (tid < kTile) S.yv[tid] = ldcg(dg + (p & 1) * kTile + tid);
            __syncthreads();
            tile_outputs_from_m<T>(S.x, S.yv, S.tmp, S.u, &S.s[0][0], a.diag + c0 * a.ldd + c0, a.ldd, w,
                                   (int)(m - c0 - w), tinvg + (p & 1) * kTile * kTile);
            signal(I);
        }
        return;
    }
    const bool helper = cta <= (unsigned)kNH;
    const int h = (int)cta - 1;
    unsigned epB = 0, epC = 0;
    for (int64_t p = 0; p < nt; ++p) {
        const int64_t c0 = p * kTile;
        const int w = tile_w(p);
        const int64_t c1 = c0 + w;
        const bool has_next = c1 < m;
        const int w2 = has_next ? tile_w(p + 1) : 0;
        const int64_t c2 = c1 + w2;
        const bool has_next2 = c2 < m;
        const int w3 = has_next2 ? tile_w(p + 2) : 0;

        if (helper) {
            if (!has_next) break;
            // rows of tile-row p+1 in column block p: Y M^T = B, X = Y D^{-1/2}
            if (!wait_count(F, (unsigned)(p + 1), a.status, &S.flag)) return;
            load_block<T>(S.x, Mg + (p & 1) * kTile * kTile, kTile, kTile, kTile);
            if (tid < kTile) S.yv[tid] = rsq<T>(ldcg(dg + (p & 1) * kTile + tid));
            __syncthreads();
            if (ty < kHelpRows) {
                const int r = h * kHelpRows + ty;
                if (r < w2) {
                    T* rp = a.diag + (c1 + r) * a.ldd + c0;
                    T y = tx < w ? ldcg(rp + tx) : T(0);
                    for (int k = 0; k < w; ++k) {
                        const T yk = __shfl_sync(0xffffffffu, y, k);
                        if (tx > k) y = fma(-yk, S.x[tx][k], y);
                    }
                    if (tx < w) rp[tx] = y * S.yv[tx];
                }
            }
            signal(H1);
            if (!wait_count(H1, (unsigned)(kNH * (p + 1)), a.status, &S.flag)) return;
            // their rows of the update of tile (p+1, p+1) with column block p
            load_block<T>(S.tmp, a.diag + c1 * a.ldd + c0, a.ldd, w2, w);
            __syncthreads();
            if (ty < kHelpRows) {
                const int rr = h * kHelpRows + ty, c = tx;
                if (rr < w2 && c <= rr) {
                    T* cp = a.diag + (c1 + rr) * a.ldd + c1 + c;
                    *cp = ldcg(cp) - dot32<T>(&S.tmp[rr][0], &S.tmp[c][0], w);
                }
            }
            signal(H2);
            // after the bulk TRSM: column block p applied to their rows of tile-row p+2
            if (!group_barrier(barB, G - 2, epB, a.status, &S.flag)) return;
            if (has_next2) {
                load_block<T>(S.s, a.diag + c2 * a.ldd + c0, a.ldd, w3, w);  // L_{p+2,p}
                __syncthreads();
                const int half = ty >> 2, rr = h * kHelpRows + (ty & 3), c = tx;
                if (rr < w3) {
                    if (half == 0 && c < w2) {  // tile (p+2, p+1)
                        T* cp = a.diag + (c2 + rr) * a.ldd + c1 + c;
                        *cp = ldcg(cp) - dot32<T>(&S.s[rr][0], &S.tmp[c][0], w);
                    } else if (half == 1 && c <= rr) {  // tile (p+2, p+2), lower
                        T* cp = a.diag + (c2 + rr) * a.ldd + c2 + c;
                        *cp = ldcg(cp) - dot32<T>(&S.s[rr][0], &S.s[c][0], w);
                    }
                }
                __threadfence();
                __syncthreads();
            }
            continue;
        }

        // ---------------- workers
        if (!wait_count(I, (unsigned)(p + 1), a.status, &S.flag)) return;
        load_block<T>(S.x, tinvg + (p & 1) * kTile * kTile, kTile, kTile, kTile);
        __syncthreads();
        // B(p): the rows below tile p except tile-row p+1 (the helpers')
        const unsigned nwk = G - kW0, wk = cta - kW0;
        const int64_t off0 = w2;
        const int64_t nrows = (m - c1) + a.r1rows + a.r2rows - off0;
        for (int64_t ch = wk; ch * 8 < nrows; ch += nwk) {
            const int64_t r = ch * 8 + ty;
            T* rp = r < nrows ? row_ptr(a, c1, off0 + r) + c0 : nullptr;
            trsm_rows<T>(S, rp, w);
        }
        if (!has_next) break;
        if (!group_barrier(barB, G - 2, epB, a.status, &S.flag)) return;

        // C(p): rank-w update of the trailing panel without tile-rows p+1, p+2
        const int64_t ntd = (m - c1 + kTile - 1) / kTile;
        const int64_t n1 = (a.r1rows + kTile - 1) / kTile, n2 = (a.r2rows + kTile - 1) / kTile;
        const int64_t tiles_d = ntd * (ntd + 1) / 2;
        const int64_t total = tiles_d + (n1 + n2) * ntd;
        const int64_t t0 = tiles_d < 3 ? tiles_d : 3;
        const T* Bpan = a.diag + c1 * a.ldd + c0;
        for (int64_t t = t0 + wk; t < total; t += nwk) {
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
            for (int i2 = 0; i2 < 2; ++i2)
#pragma unroll
                for (int j2 = 0; j2 < 2; ++j2) {
                    const int r = cy + 16 * i2, c = cx + 16 * j2;
                    if (r < rows && c < cols) {
                        T* cp = Cbase + (int64_t)r * ldc + cj * kTile + c;
                        *cp = ldcg(cp) - acc[i2][j2];
                    }
                }
            __syncthreads();
        }
        if (!group_barrier(barC, G - kW0, epC, a.status, &S.flag)) return;
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
    if (G < kW0 + 8) return cudaErrorNotSupported;  // too few SMs: callers use the launch-based sweep
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
    a.scratch = tinv;
    a.info = info;
    a.row0 = info_row0;
    a.bar = bar;
    a.status = status;
    e = cudaMemsetAsync(bar, 0, 8 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    void* args[] = {(void*)&a};
    prof_before(s);
    e = cudaLaunchCooperativeKernel((const void*)k_factor_panel<T>, dim3(G), dim3(NT), args, 0, s);
    // useful flops: Cholesky of the m x m block + TRSM of the rows below it
    const double md = (double)m;
    prof_after(SGB_KCLASS_PANEL, s, md * md * md / 3.0 + (double)(a.r1rows + a.r2rows) * md * md);
    return e;
}

template cudaError_t factor_panel_persistent<double>(double*, int64_t, int64_t, RowSet<double>, RowSet<double>,
                                                     double*, unsigned*, int32_t*, int32_t*, int64_t,
                                                     cudaStream_t);
template cudaError_t factor_panel_persistent<float>(float*, int64_t, int64_t, RowSet<float>, RowSet<float>,
                                                    float*, unsigned*, int32_t*, int32_t*, int64_t, cudaStream_t);

}  // namespace sgb
