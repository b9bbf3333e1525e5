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
//                pipeline of factor_tile_m), whose warp 4 publishes the
//                columns of M, d and d^{-1/2} as they are produced
//                (counter of published columns), then counter F at the end
//                of the tile; tile p+1 arrives by value from the helpers;
//   CTAs 1..kNH  helpers: the rows of tile-row p+1 in column block p by
//                unit-triangular substitution (Y M^T = B, X = Y D^{-1/2}),
//                following the published columns, handed to each other by
//                value; then their rows of the update of tile (p+1, p+1),
//                handed to the factorizer by value; after barrier B they
//                apply column block p to their rows of tile-row p+2 (tiles
//                (p+2, p+1) and (p+2, p+2)), so nothing the next step needs
//                waits for the bulk update;
//   CTA kNH+1    L writer: from M_p, d_p the tile's L into the matrix
//                (counter I);
//   CTAs kNH+2.. workers: warps 0-3 the other rows below tile p (and, with
//                xinv, the rows of L^{-T}), each first given its share of
//                the trailing update of step p-1 (column block p-1 on its
//                column block p), then the same substitution following the
//                published columns; warps 4-7 meanwhile the rest of the
//                trailing update of step p-1 (the next tile's operands and
//                C loaded during the current tile's FMAs), then they take
//                rows too (a per-CTA row counter); barrier B (with the
//                helpers).
//
// M, d and d^{-1/2} rotate through three buffers; the factorizer waits for
// the L writer before overwriting one.  The two hand-offs on the chain from
// one diagonal tile to the next go by value through staging buffers (a
// sentinel NaN until the producer stores the value, see Staged<T>), so no
// fence or counter sits between producer and consumer; the factorizer
// resets each staging buffer once its consumers are provably done.  Every
// other wait is a bounded poll of a word in global memory: one that does
// not complete within the limit sets the status word to SGB_ERR_TIMEOUT
// and the CTA leaves (the cooperative launch guarantees that all CTAs are
// resident, so no wait depends on an unscheduled CTA).  Data produced by
// other CTAs is read with ld.global.cg (L2) or relaxed GPU-scope loads,
// never from a possibly stale L1 line.
#include <math.h>

#include "sgb_internal.cuh"
#include "sgb_tile.cuh"

namespace sgb {

namespace {

constexpr int NT = 256;
constexpr int kNH = 8;                 // helper CTAs of the next diagonal tile
constexpr int kHelpRows = kTile / kNH;  // rows of a tile-row per helper
constexpr int kInv = kNH + 1;           // the L writer CTA
constexpr int kW0 = kNH + 2;            // first worker CTA

template <typename T>
struct PanelArgs {
    T* diag;
    int64_t m, ldd;
    T* r1;
    int64_t r1rows, r1ld;
    T* r2;
    int64_t r2rows, r2ld;
    T* xinv;  // m x m, row-major (ld xld): L^{-T} out, or null
    int64_t xld;
    T* scratch;  // [3][32][32] M^T by column, [3][32] d, [3][32] d^{-1/2},
                 // [2][32][32] staged diagonal tiles, [2][32][32] staged tile-rows,
                 // [3][32 * 32 + 32] staged columns of M and d
    int32_t* info;
    int64_t row0;
    unsigned* bar;    // [0] F, [1] I, [4] barrier B, [8] columns of M
                      // published; zero at launch
    int32_t* status;  // SGB_ERR_TIMEOUT on a stuck wait
    long long spin;   // poll limit of every bounded wait
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

// Barrier over `nblocks` CTAs on a monotonic arrival counter: barrier
// number e (1, 2, ...) completes when the counter reaches e * nblocks.
// Arrivals are fire-and-forget reductions, so no CTA waits for an atomic's
// return.  Returns false (on every thread of the CTA) if it timed out.
__device__ __forceinline__ bool group_barrier(unsigned* cnt, unsigned nblocks, unsigned& epoch, int32_t* status,
                                              int* sflag, long long spin) {
    __syncthreads();
    if (threadIdx.x == 0) {
        epoch += 1;
        const unsigned target = epoch * nblocks;
        int ok = 1;
        __threadfence();
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(cnt) : "memory");
        long long spins = 0;
        while ((int)(ld_acquire(cnt) - target) < 0) {
            if (++spins > spin || status_bad(status)) {
                ok = 0;
                atomicExch(status, SGB_ERR_TIMEOUT);
                break;
            }
            __nanosleep(32);
        }
        *sflag = ok && !status_bad(status);
    }
    __syncthreads();
    return *sflag != 0;
}

// Wait until *ctr >= target (tight poll: only a few CTAs wait here); false
// (on every thread) on a timeout or an error raised elsewhere.
__device__ __forceinline__ bool wait_count(const unsigned* ctr, unsigned target, int32_t* status, int* sflag,
                                           long long spin) {
    if (threadIdx.x == 0) {
        long long spins = 0;
        int ok = 1;
        while (ld_acquire(ctr) < target) {
            if (++spins > spin || status_bad(status)) {
                ok = 0;
                atomicExch(status, SGB_ERR_TIMEOUT);
                break;
            }
        }
        *sflag = ok;
    }
    __syncthreads();
    return *sflag != 0;
}

// CTA-uniform check of the status word (also a CTA barrier).
__device__ __forceinline__ bool cta_ok(const int32_t* status, int* sflag) {
    __syncthreads();
    if (threadIdx.x == 0) *sflag = !status_bad(status);
    __syncthreads();
    return *sflag != 0;
}

// Named barrier `id` over the first `nthreads` threads' warps (a group of
// warps synchronizing without the rest of the CTA).
__device__ __forceinline__ void group_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Publish: make this CTA's global writes visible, then count on ctr (the
// barrier orders the CTA's writes before thread 0's fence, which is
// cumulative).
__device__ __forceinline__ void signal(unsigned* ctr) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ctr, 1u);
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

// One row per warp: row <- row * L^{-T} over the w columns of the row
// pointer, with L = M diag(d)^{1/2}: Y M^T = row by substitution (lane =
// column; one shuffle and one FMA per column), X = Y diag(d)^{-1/2}.  The
// columns of M (transposed in mt) and d^{-1/2} (rv) are consumed as the
// factorizer publishes them: column k once *colcount >= col_base + k + 1
// (bounded wait; `sleep` backs off between polls), all available columns
// loaded at once.  With stage_row the result also goes to that staging row
// (hand-off by value).  With unit >= 0
// the row is the unit vector e_unit instead of the stored values (a row of
// the identity, whose solve is a row of L^{-T}); with preset the row starts
// from y0 (lane = column) instead.  Returns false on a timeout or an error
// raised elsewhere.
template <typename T>
__device__ __forceinline__ bool trsm_row_pipe(T* rp, int w, const T* mt, const T* rv, const unsigned* colcount,
                                              unsigned col_base, int32_t* status, bool sleep, long long spin,
                                              int unit = -1, T* stage_row = nullptr, bool preset = false,
                                              T y0 = T(0)) {
    const int tx = threadIdx.x & 31;
    T y = tx < w ? (unit >= 0 ? T(tx == unit ? 1 : 0) : preset ? y0 : ldcg(rp + tx)) : T(0);
    T r = T(0);
    int k = 0;
    long long spins = 0;
    while (k < w) {
        int avail = 0;
        if (tx == 0) {
            for (;;) {
                const unsigned c = ld_acquire(colcount);
                avail = c > col_base ? (int)(c - col_base) : 0;
                if (avail > k) break;
                if (++spins > spin || status_bad(status)) {
                    atomicExch(status, SGB_ERR_TIMEOUT);
                    avail = -1;
                    break;
                }
                if (sleep) __nanosleep(32);
            }
        }
        avail = __shfl_sync(0xffffffffu, avail, 0);
        if (avail < 0) return false;
        if (avail > w) avail = w;
        while (k < avail) {
            const int nb = (avail - k) < kTile ? (avail - k) : kTile;
            T mk[kTile];
#pragma unroll
            for (int u = 0; u < kTile; ++u) mk[u] = u < nb ? ldcg(mt + (k + u) * kTile + tx) : T(0);
            if (tx >= k && tx < k + nb) r = ldcg(rv + tx);
#pragma unroll
            for (int u = 0; u < kTile; ++u) {
                if (u < nb) {
                    const T yk = __shfl_sync(0xffffffffu, y, k + u);
                    if (tx > k + u) y = fma(-yk, mk[u], y);
                }
            }
            k += nb;
        }
    }
    if (tx < w) {
        const T x = y * r;
        rp[tx] = x;
        if (stage_row != nullptr) stage_put(stage_row + tx, x);
    }
    return true;
}

// The helpers' rows: as trsm_row_pipe, with the columns of M and the pivots
// taken by value from the factorizer's staging buffer vc ([32][32] M^T by
// column, then [32] d) as they land -- no counter, no fence in between.
// Up to eight columns are polled at once; the leading ones every lane holds
// are applied.  d^{-1/2} is formed here, lane by lane, as the pivots
// arrive.  The result also goes to the staging row.  Returns false on a
// timeout or an error raised elsewhere.
template <typename T>
__device__ __forceinline__ bool trsm_row_vals(T* rp, int w, const T* vc, int32_t* status, T* stage_row,
                                              long long spin) {
    const int tx = threadIdx.x & 31;
    T y = tx < w ? ldcg(rp + tx) : T(0);
    T r = T(0);
    int k = 0;
    long long rounds = 0;
    while (k < w) {
        const int nb = (w - k) < 8 ? (w - k) : 8;
        decltype(Staged<T>::ld(vc)) raw[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) raw[u] = u < nb ? Staged<T>::ld(vc + (k + u) * kTile + tx) : Staged<T>::kSentinel;
        // this lane's pivot in the same round (staged before its column;
        // polled below only if it has not landed yet)
        const auto rd = (tx >= k && tx < k + nb) ? Staged<T>::ld(vc + kTile * kTile + tx) : Staged<T>::kSentinel;
        int navail = 0;
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (navail == u && u < nb && __all_sync(0xffffffffu, raw[u] != Staged<T>::kSentinel)) navail = u + 1;
        if (navail == 0) {
            if (++rounds > spin || ((rounds & 63) == 0 && status_bad(status))) {
                atomicExch(status, SGB_ERR_TIMEOUT);
                return false;
            }
            continue;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (u < navail) {
                const T yk = __shfl_sync(0xffffffffu, y, k + u);
                if (tx > k + u) y = fma(-yk, Staged<T>::val(raw[u]), y);
            }
        }
        if (tx >= k && tx < k + navail) {
            T d;
            if (rd != Staged<T>::kSentinel) {
                d = Staged<T>::val(rd);
            } else {
                const T* dp[1] = {vc + kTile * kTile + tx};
                const bool want[1] = {true};
                T dv[1];
                if (!stage_take<T, 1>(dp, want, dv, spin, status)) atomicExch(status, SGB_ERR_TIMEOUT);
                d = dv[0];
            }
            r = rsq<T>(d);
        }
        k += navail;
    }
    if (tx < w) {
        const T x = y * r;
        rp[tx] = x;
        stage_put(stage_row + tx, x);
    }
    return true;
}

// dst[32 x 32] <- rows x cols block of a row-major source (zero padded);
// each thread issues its four loads before storing any.
template <typename T>
__device__ __forceinline__ void load_block(T (*dst)[kTile + 1], const T* src, int64_t ld, int rows, int cols) {
    constexpr int U = kTile * kTile / NT;
    T v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int e = threadIdx.x + u * NT, r = e / kTile, c = e % kTile;
        v[u] = (r < rows && c < cols) ? ldcg(src + (int64_t)r * ld + c) : T(0);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int e = threadIdx.x + u * NT;
        dst[e / kTile][e % kTile] = v[u];
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
    // the next kernel in the stream (a programmatic dependent launch) may
    // start launching now; it waits for this grid's completion before it
    // touches memory
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    unsigned* F = a.bar + 0;
    unsigned* I = a.bar + 1;
    unsigned* barB = a.bar + 4;
    unsigned* CC = a.bar + 8;
    T* Mg = a.scratch;                      // [3][32*32], column k of M at [k][0..31]
    T* dg = a.scratch + 3 * kTile * kTile;  // [3][32] d
    T* rg = dg + 3 * kTile;                 // [3][32] d^{-1/2}
    T* stT = rg + 3 * kTile;                // [2][32*32] tile (p, p) after its last update, by value
    T* stL = stT + 2 * kTile * kTile;       // [2][32*32] tile-row p+1 in column block p, by value
    constexpr int kVc = kTile * kTile + kTile;
    T* stV = stL + 2 * kTile * kTile;       // [3][32*32 + 32] columns of M and d of tile p, by value
    auto tile_w = [&](int64_t p) -> int { return (int)((m - p * kTile) < kTile ? (m - p * kTile) : kTile); };

    if (cta == 0) {
        // ---------------- factorizer
        // staging buffers to the sentinel before the first column is
        // published (every later hand-off is ordered after it)
        for (int e = tid; e < 4 * kTile * kTile + 3 * kVc; e += NT) stage_clear(stT + e);
        __syncthreads();
        for (int64_t p = 0; p < nt; ++p) {
            const int64_t c0 = p * kTile;
            const int w = tile_w(p);
            if (p >= 3 && !wait_count(I, (unsigned)(p - 2), a.status, &S.flag, a.spin)) return;  // buffer p % 3 free
            const int buf = (int)(p % 3);
            // tile p >= 1 arrives by value from the helpers (their update
            // with column block p-1); tile-row staging p-1 is then free
            factor_tile_m<T>(S, a.diag + c0 * a.ldd + c0, a.ldd, w, a.info, a.row0 + c0, Mg + buf * kTile * kTile,
                             dg + buf * kTile, rg + buf * kTile, CC, (unsigned)(p * kTile),
                             p >= 1 ? stT + (p & 1) * kTile * kTile : nullptr,
                             p >= 1 ? stL + ((p - 1) & 1) * kTile * kTile : nullptr, a.status, stV + (p % 3) * kVc,
                             p >= 1 ? stV + ((p - 1) % 3) * kVc : nullptr, a.spin);
            if (!cta_ok(a.status, &S.flag)) return;
            signal(F);
        }
        return;
    }
    if (cta == (unsigned)kInv) {
        // ---------------- L writer
        for (int64_t p = 0; p < nt; ++p) {
            const int64_t c0 = p * kTile;
            const int w = tile_w(p);
            if (!wait_count(F, (unsigned)(p + 1), a.status, &S.flag, a.spin)) return;
            const int buf = (int)(p % 3);
            {
                const T* mt = Mg + buf * kTile * kTile;
                for (int e = tid; e < kTile * kTile; e += NT) S.x[e % kTile][e / kTile] = ldcg(mt + e);
            }
            if (tid < kTile) {
                S.yv[tid] = ldcg(dg + buf * kTile + tid);
                S.tmp[0][tid] = ldcg(rg + buf * kTile + tid);
            }
            __syncthreads();
            tile_l_from_m<T>(S.x, S.yv, &S.tmp[0][0], a.diag + c0 * a.ldd + c0, a.ldd, w, (int)(m - c0 - w));
            signal(I);
        }
        return;
    }
    const bool helper = cta <= (unsigned)kNH;
    const int h = (int)cta - 1;
    unsigned epB = 0;
    if (tid == 0) S.rowq[0] = S.rowq[1] = 0;
    __syncthreads();
    for (int64_t p = 0; p < nt; ++p) {
        const int64_t c0 = p * kTile;
        const int w = tile_w(p);
        const int64_t c1 = c0 + w;
        const bool has_next = c1 < m;
        const int w2 = has_next ? tile_w(p + 1) : 0;
        const int64_t c2 = c1 + w2;
        const bool has_next2 = c2 < m;
        const int w3 = has_next2 ? tile_w(p + 2) : 0;
        const T* Mp = Mg + (p % 3) * kTile * kTile;
        const T* rp3 = rg + (p % 3) * kTile;

        if (helper) {
            if (!has_next) break;
            // rows of tile-row p+1 in column block p (Y M^T = B, X = Y D^{-1/2}),
            // column by column as the factorizer publishes M; a timeout sets
            // the status word, which the wait below sees
            T* sL = stL + (p & 1) * kTile * kTile;
            // The staging buffers of this step were reset during tiles p-2
            // (columns) and p-1 (tile-row), each ordered before tile p's
            // first published columns: acquire those before any poll.
            if (!wait_count(CC, (unsigned)(p * kTile + 1), a.status, &S.flag, a.spin)) return;
            if (ty < kHelpRows) {
                const int r = h * kHelpRows + ty;
                if (r < w2)
                    trsm_row_vals<T>(a.diag + (c1 + r) * a.ldd + c0, w, stV + (p % 3) * kVc, a.status, sL + r * kTile,
                                     a.spin);
            }
            // this thread's element of tile (p+1, p+1) (last written by this CTA)
            const int rr1 = h * kHelpRows + ty, cc1 = tx;
            const bool own1 = ty < kHelpRows && rr1 < w2 && cc1 <= rr1;
            const T cold = own1 ? ldcg(a.diag + (c1 + rr1) * a.ldd + c1 + cc1) : T(0);
            // all of tile-row p+1 by value from the helpers, then their rows
            // of the update of tile (p+1, p+1), handed to the factorizer by value
            {
                constexpr int U = kTile * kTile / NT;
                const T* sp[U];
                bool want[U];
                T v[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int e = tid + u * NT;
                    sp[u] = sL + e;
                    want[u] = e / kTile < w2 && e % kTile < w;
                }
                const bool took = stage_take<T, U>(sp, want, v, a.spin, a.status);
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int e = tid + u * NT;
                    S.tmp[e / kTile][e % kTile] = want[u] ? v[u] : T(0);
                }
                if (__syncthreads_or(!took)) {
                    if (tid == 0) atomicExch(a.status, SGB_ERR_TIMEOUT);
                    return;
                }
            }
            if (own1)
                stage_put(stT + ((p + 1) & 1) * kTile * kTile + rr1 * kTile + cc1,
                          cold - dot32<T>(&S.tmp[rr1][0], &S.tmp[cc1][0], w));
            // after the bulk TRSM: column block p applied to their rows of tile-row p+2
            if (!group_barrier(barB, G - 2, epB, a.status, &S.flag, a.spin)) return;
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
        // Step p, two groups of four warps side by side:
        //   warps 0-3  B(p): the rows below tile p except tile-row p+1 (the
        //              helpers'), and with xinv the rows of L^{-T} not zero
        //              in column block p (rows < c1; those of tile-row p
        //              start as identity rows), one row at a time per
        //              warp: first column block p-1 applied to the row's
        //              column block p
        //              (its share of the trailing update of step p-1),
        //              then the substitution following the published
        //              columns of M;
        //   warps 4-7  the rest of that trailing update: column block p-1
        //              on the trailing panel of step p-1 without tile-rows
        //              p, p+1 and without column block p; then rows as well
        //              in tall panels.
        // Then barrier B (with the helpers).  The rows never wait for the
        // bulk update, and the bulk update runs while the rows follow the
        // pivots.
        const unsigned nwk = G - kW0, wk = cta - kW0;
        const bool prev = p >= 1;  // the trailing update of step p-1 is due
        const int64_t off0 = w2;
        const int64_t nbase = (m - c1) + a.r1rows + a.r2rows - off0;
        const int64_t nrows = nbase + (a.xinv ? c1 : 0);
        if (tid == 0) S.rowq[(p + 1) & 1] = 0;  // the next step's row counter (used after barrier B)
        // This CTA's q-th row of the step: wk*4 + (q & 3) + (q / 4) * nwk*4.
        // Warps 0-3 start with q = ty and take every further q from a shared
        // counter; when the rows outnumber the first round (the tall panels
        // of the FP64 forms), warps 4-7 join once their share of the update
        // is done, with their own copy of the tile-row operand.
        const bool tall = nrows > (int64_t)nwk * 4;
        // tile-row p in column block p-1 (the helpers' rows of step p-1),
        // the operand of every row's share of the update: to S.x (warps
        // 0-3) or S.u (warps 4-7)
        auto load_tile_row = [&](T (*dst)[kTile + 1], int gt) {
            for (int e = gt; e < kTile * kTile; e += 128) {
                const int r = e / kTile, k = e % kTile;
                dst[r][k] = r < w ? ldcg(a.diag + (c0 + r) * a.ldd + (c0 - kTile) + k) : T(0);
            }
        };
        auto row_of = [&](int64_t q) { return (int64_t)wk * 4 + (q & 3) + (q >> 2) * (int64_t)nwk * 4; };
        auto next_q = [&]() -> int64_t {
            int g = 0;
            if (tx == 0) g = atomicAdd(&S.rowq[p & 1], 1);
            return 4 + (int64_t)__shfl_sync(0xffffffffu, g, 0);
        };
        auto do_row = [&](int64_t r, T (*tr)[kTile + 1]) -> bool {
            T* rp;
            int unit = -1;
            bool fresh = false;  // L^{-T} tile-row p-1: column block p not written yet
            if (r < nbase) {
                rp = row_ptr(a, c1, off0 + r) + c0;
            } else {
                const int64_t xr = r - nbase;
                rp = a.xinv + xr * a.xld + c0;
                if (xr >= c0) unit = (int)(xr - c0);
                else fresh = xr >= c0 - kTile;
            }
            T y0 = T(0);
            if (prev && unit < 0) {  // y0 = row(block p) - row(block p-1) * (tile-row p of block p-1)^T
                const T av = ldcg(rp - kTile + tx);
                y0 = (fresh || tx >= w) ? T(0) : ldcg(rp + tx);
#pragma unroll
                for (int k = 0; k < kTile; ++k) y0 = fma(-__shfl_sync(0xffffffffu, av, k), tr[tx][k], y0);
            }
            return trsm_row_pipe<T>(rp, w, Mp, rp3, CC, (unsigned)(p * kTile), a.status, true, a.spin, unit, nullptr,
                                    prev && unit < 0, y0);
        };
        if (ty < 4) {
            if (prev) {
                load_tile_row(S.x, tid);
                group_sync(1, 128);
            }
            for (int64_t q = ty;; q = next_q()) {
                const int64_t r = row_of(q);
                if (r >= nrows || !do_row(r, S.x)) break;
            }
        } else if (prev) {
            // step q = p-1: column block q, trailing panel from c1q = c0
            const int64_t c0q = c0 - kTile, c1q = c0;
            const int64_t ntd = (m - c1q + kTile - 1) / kTile;  // tile-rows from tile-row p
            const int64_t n1 = (a.r1rows + kTile - 1) / kTile, n2 = (a.r2rows + kTile - 1) / kTile;
            const int64_t nx = a.xinv ? p : 0;  // tile-rows of L^{-T} not zero in block q
            // D tiles (ti, cj) with ti >= 2 and 1 <= cj <= ti, then the tiles
            // of the other row sets with cj >= 1
            const int64_t tiles_d = ntd >= 2 ? ntd * (ntd - 1) / 2 - 1 : 0;
            const int64_t total = ntd >= 2 ? tiles_d + (n1 + n2 + nx) * (ntd - 1) : 0;
            const T* Bpan = a.diag + c1q * a.ldd + c0q;
            struct TileRef {
                T* C;
                const T* A;
                int64_t ldc, rows, cols, cj;
                bool fresh;  // C holds no value yet (L^{-T} tile-row q): C = -update
            };
            auto tile_ref = [&](int64_t t) {
                TileRef R;
                R.fresh = false;
                int64_t ti;
                if (t < tiles_d) {  // (ti - 1, cj - 1) over the triangle of ntd - 1 tile-rows, from its second tile
                    const int64_t tt = t + 1;
                    int64_t ui = (int64_t)((sqrt(8.0 * (double)tt + 1.0) - 1.0) * 0.5);
                    while (ui * (ui + 1) / 2 > tt) --ui;
                    while ((ui + 1) * (ui + 2) / 2 <= tt) ++ui;
                    ti = ui + 1;
                    R.cj = tt - ui * (ui + 1) / 2 + 1;
                    R.C = a.diag + (c1q + ti * kTile) * a.ldd + c1q;
                    R.A = a.diag + (c1q + ti * kTile) * a.ldd + c0q;
                    R.ldc = a.ldd;
                    R.rows = (m - c1q) - ti * kTile;
                } else {
                    const int64_t u = t - tiles_d;
                    const int64_t set = u / (ntd - 1);
                    R.cj = 1 + u % (ntd - 1);
                    if (set < n1) {
                        ti = set;
                        R.C = a.r1 + ti * kTile * a.r1ld + c1q;
                        R.A = a.r1 + ti * kTile * a.r1ld + c0q;
                        R.ldc = a.r1ld;
                        R.rows = a.r1rows - ti * kTile;
                    } else if (set < n1 + n2) {
                        ti = set - n1;
                        R.C = a.r2 + ti * kTile * a.r2ld + c1q;
                        R.A = a.r2 + ti * kTile * a.r2ld + c0q;
                        R.ldc = a.r2ld;
                        R.rows = a.r2rows - ti * kTile;
                    } else {
                        ti = set - n1 - n2;
                        R.C = a.xinv + ti * kTile * a.xld + c1q;
                        R.A = a.xinv + ti * kTile * a.xld + c0q;
                        R.ldc = a.xld;
                        R.rows = m - ti * kTile;
                        R.fresh = ti == p - 1;
                    }
                }
                if (R.rows > kTile) R.rows = kTile;
                R.cols = (m - c1q) - R.cj * kTile;
                if (R.cols > kTile) R.cols = kTile;
                return R;
            };
            // 128 threads, 8 outputs each: rows cy + 8 i (i < 4), columns cx + 16 j (j < 2)
            const int gt = tid - 128, cx = gt & 15, cy = gt >> 4;
            constexpr int U = kTile * kTile / 128;
            T va[U], vb[U], vc[4][2];
            auto fetch = [&](const TileRef& R) {
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int e = gt + u * 128, r = e / kTile, k = e % kTile;
                    va[u] = r < R.rows ? ldcg(R.A + (int64_t)r * R.ldc + k) : T(0);
                    vb[u] = r < R.cols ? ldcg(Bpan + (R.cj * kTile + r) * a.ldd + k) : T(0);
                }
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        const int r = cy + 8 * i, c = cx + 16 * j;
                        vc[i][j] = (!R.fresh && r < R.rows && c < R.cols)
                                       ? ldcg(R.C + (int64_t)r * R.ldc + R.cj * kTile + c)
                                       : T(0);
                    }
            };
            int64_t t = wk;
            TileRef cur;
            if (t < total) {
                cur = tile_ref(t);
                fetch(cur);
            }
            for (; t < total; t += nwk) {
                group_sync(2, 128);  // the previous tile's operands are no longer read
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int e = gt + u * 128;
                    S.s[e / kTile][e % kTile] = va[u];
                    S.tmp[e / kTile][e % kTile] = vb[u];
                }
                T acc[4][2];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 2; ++j) acc[i][j] = vc[i][j];
                group_sync(2, 128);
                const TileRef now = cur;
                if (t + nwk < total) {  // next tile's operands in flight during this tile's FMAs
                    cur = tile_ref(t + nwk);
                    fetch(cur);
                }
                for (int k = 0; k < kTile; ++k) {
                    T av[4], bv[2];
#pragma unroll
                    for (int i = 0; i < 4; ++i) av[i] = S.s[cy + 8 * i][k];
#pragma unroll
                    for (int j = 0; j < 2; ++j) bv[j] = S.tmp[cx + 16 * j][k];
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 2; ++j) acc[i][j] = fma(-av[i], bv[j], acc[i][j]);
                }
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        const int r = cy + 8 * i, c = cx + 16 * j;
                        if (r < now.rows && c < now.cols) now.C[(int64_t)r * now.ldc + now.cj * kTile + c] = acc[i][j];
                    }
            }
        }
        if (ty >= 4 && tall) {  // the update's share done: help with the rows still left
            if (prev) {
                load_tile_row(S.u, tid - 128);
                group_sync(2, 128);
            }
            for (;;) {
                const int64_t r = row_of(next_q());
                if (r >= nrows || !do_row(r, S.u)) break;
            }
        }
        if (!has_next) break;
        if (!group_barrier(barB, G - 2, epB, a.status, &S.flag, a.spin)) return;
    }
}

int g_panel_grid[64] = {};

}  // namespace

template <typename T>
cudaError_t factor_panel_persistent(T* diag, int64_t m, int64_t ldd, RowSet<T> r1, RowSet<T> r2, T* tinv,
                                    unsigned* bar, int32_t* status, int32_t* info, int64_t info_row0,
                                    cudaStream_t s, T* xinv, int grid_cap) {
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
    const int G = (grid_cap > 0 && grid_cap < g_panel_grid[dev]) ? grid_cap : g_panel_grid[dev];
    if (G < kW0 + 8) return cudaErrorNotSupported;  // too few CTAs: callers use the launch-based sweep
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
    a.xinv = xinv;
    a.xld = m;
    a.scratch = tinv;
    a.info = info;
    a.row0 = info_row0;
    a.bar = bar;
    a.status = status;
    a.spin = spin_limit();
    e = cudaMemsetAsync(bar, 0, 16 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    void* args[] = {(void*)&a};
    prof_before(s, SGB_KCLASS_PANEL);
    e = cudaLaunchCooperativeKernel((const void*)k_factor_panel<T>, dim3(G), dim3(NT), args, 0, s);
    // useful flops: Cholesky of the m x m block + TRSM of the rows below it
    // (+ the triangular inverse)
    const double md = (double)m;
    prof_after(SGB_KCLASS_PANEL, s,
               md * md * md / 3.0 * (xinv ? 2.0 : 1.0) + (double)(a.r1rows + a.r2rows) * md * md);
    return e;
}

template cudaError_t factor_panel_persistent<double>(double*, int64_t, int64_t, RowSet<double>, RowSet<double>,
                                                     double*, unsigned*, int32_t*, int32_t*, int64_t, cudaStream_t,
                                                     double*, int);
template cudaError_t factor_panel_persistent<float>(float*, int64_t, int64_t, RowSet<float>, RowSet<float>,
                                                    float*, unsigned*, int32_t*, int32_t*, int64_t, cudaStream_t,
                                                    float*, int);

namespace {
thread_local int t_capture_panel_grid = 0;
}
void set_capture_panel_grid(int ctas) { t_capture_panel_grid = ctas < 0 ? 0 : ctas; }
int capture_panel_grid() { return t_capture_panel_grid; }

namespace {
thread_local bool t_capture_tc_split = false;
}
void set_capture_tc_split(bool on) { t_capture_tc_split = on; }
bool capture_tc_split() { return t_capture_tc_split; }

}  // namespace sgb
