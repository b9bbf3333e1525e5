// Diagonal-tile kernels shared by the launch-based sweep (sgb_potrf.cu)
// and the persistent column-block kernel (sgb_panel.cu): Cholesky of one
// <= 32 x 32 tile with a one-column lookahead, and the tile's inverse by
// recursive doubling.  One CTA of kTileThreads threads runs a tile.
#pragma once

#include <math.h>

#include "sgb_internal.cuh"

namespace sgb {

constexpr int kTileThreads = 256;

// Positive, finite and not subnormal: checked on the bits, so the pivot
// test costs no FP64 instruction (each one occupies an SM quarter's FP64
// unit for ~64 cycles on this part).
__device__ __forceinline__ bool pivot_ok(double d) {
    const long long bits = __double_as_longlong(d);
    const int ex = (int)((bits >> 52) & 0x7ff);
    return bits > 0 && ex != 0 && ex != 0x7ff;
}
__device__ __forceinline__ bool pivot_ok(float d) {
    const int bits = __float_as_int(d);
    const int ex = (bits >> 23) & 0xff;
    return bits > 0 && ex != 0 && ex != 0xff;
}

template <typename T>
__device__ __forceinline__ T rsq(T x);
template <>
__device__ __forceinline__ double rsq<double>(double x) { return rsqrt(x); }
template <>
__device__ __forceinline__ float rsq<float>(float x) { return rsqrtf(x); }

template <typename T>
struct Smem {
    T s[kTile][kTile + 1];
    T x[kTile][kTile + 1];
    T tmp[kTile][kTile + 1];
    T u[kTile][kTile + 1];
    T yv[kTile];
    unsigned short tri[kTile * (kTile + 1) / 2];  // (row << 8) | col of the lower triangle, row-major
    int fail;
    int flag;
    int pub;      // factor_tile_m: columns the companion has completed
    int rowq[2];  // column-block kernel workers: row counters of alternate steps
};

// Recursive-doubling inverse of the (identity padded) lower tile s into x.
template <typename T>
__device__ void tile_inverse_dev(Smem<T>& S) {
    // Recursive doubling from 4 x 4 leaves.  Every phase computes at most one
    // output per thread, as a dot product split over four independent
    // accumulators, so the dependent FP64 chain per phase is short (each FP64
    // warp instruction occupies its SM quarter for ~64 cycles on this part).
    const int tid = threadIdx.x;
    for (int e = tid; e < kTile * kTile; e += kTileThreads) S.x[e / kTile][e % kTile] = T(0);
    __syncthreads();
    if (tid < 32) {  // eight 4 x 4 leaves, one column per thread
        const int b0 = (tid >> 2) * 4, j = tid;
        for (int r = j; r < b0 + 4; ++r) {
            T sum = (r == j) ? T(1) : T(0);
            for (int k = j; k < r; ++k) sum = fma(-S.s[r][k], S.x[k][j], sum);
            S.x[r][j] = sum * S.yv[r];
        }
    }
    __syncthreads();
#pragma unroll 1
    for (int h = 4; h < kTile; h *= 2) {  // block size h -> 2h
        const int nout = (kTile / (2 * h)) * h * h;  // <= 256
        int r = 0, c = 0, o = 0;
        if (tid < nout) {
            const int bi = tid / (h * h), rem = tid % (h * h);
            r = rem / h;
            c = rem % h;
            o = bi * 2 * h;
            // tmp = L21 X11 (X11 lower triangular: k >= c)
            const T* lr = &S.s[o + h + r][o];
            T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
            int k = c;
            for (; k + 3 < h; k += 4) {
                a0 = fma(lr[k], S.x[o + k][o + c], a0);
                a1 = fma(lr[k + 1], S.x[o + k + 1][o + c], a1);
                a2 = fma(lr[k + 2], S.x[o + k + 2][o + c], a2);
                a3 = fma(lr[k + 3], S.x[o + k + 3][o + c], a3);
            }
            for (; k < h; ++k) a0 = fma(lr[k], S.x[o + k][o + c], a0);
            S.tmp[o + h + r][o + c] = (a0 + a1) + (a2 + a3);
        }
        __syncthreads();
        if (tid < nout) {
            // X21 = -X22 tmp (X22 lower triangular: k <= r)
            const T* xr = &S.x[o + h + r][o + h];
            T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
            int k = 0;
            for (; k + 3 <= r; k += 4) {
                a0 = fma(xr[k], S.tmp[o + h + k][o + c], a0);
                a1 = fma(xr[k + 1], S.tmp[o + h + k + 1][o + c], a1);
                a2 = fma(xr[k + 2], S.tmp[o + h + k + 2][o + c], a2);
                a3 = fma(xr[k + 3], S.tmp[o + h + k + 3][o + c], a3);
            }
            for (; k <= r; ++k) a0 = fma(xr[k], S.tmp[o + h + k][o + c], a0);
            S.x[o + h + r][o + c] = -((a0 + a1) + (a2 + a3));
        }
        __syncthreads();
    }
}

// Reciprocal of a positive, normal pivot with the FP64 chain cut to three
// dependent instructions: a 20-bit seed from the approximate FP64
// reciprocal instruction (measured on this part over 4M random normal
// inputs: relative error <= 2^-19.9), then the truncated series
// 1/d = r0 (1 + e + e^2 + ...), e = 1 - d r0 (Markstein / Goldschmidt
// refinement), whose e^3 ~ 2^-60 term is below half an ulp (the same
// inputs: <= 2^-52 relative after refinement).  Pivots whose reciprocal
// would be subnormal (d >= 2^1021; the approximation flushes those) take
// the IEEE division; the branch is uniform because every lane holds the
// same pivot.
__device__ __forceinline__ double rcp_pivot(double d) {
    if (((__double2hiint(d) >> 20) & 0x7ff) > 2044) return 1.0 / d;
    double r0;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r0) : "d"(d));
    const double e = fma(-d, r0, 1.0);
    const double t = fma(e, e, e);
    return fma(r0, t, r0);
}
__device__ __forceinline__ float rcp_pivot(float d) { return 1.0f / d; }

// Named barriers of the pivot/worker pipeline (ids 1-4; 0 is __syncthreads).
__device__ __forceinline__ void nbar_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void nbar_arrive(int id, int n) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Hand-off by value: a staging element holds a signaling NaN whose payload
// no arithmetic produces (results are canonical quiet NaNs) until its
// producer stores the real value with a relaxed GPU-scope store; the
// consumer polls the element itself, so no fence and no counter sit
// between them.  Single-copy atomicity of aligned 4- and 8-byte accesses
// makes the poll see either the sentinel or the whole value.
template <typename T>
struct Staged;
template <>
struct Staged<double> {
    static constexpr unsigned long long kSentinel = 0x7FF0DEADBEEF5EB1ull;
    static __device__ __forceinline__ unsigned long long ld(const double* p) {
        unsigned long long v;
        asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
        return v;
    }
    static __device__ __forceinline__ void st(double* p, unsigned long long v) {
        asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
    }
    static __device__ __forceinline__ double val(unsigned long long v) { return __longlong_as_double((long long)v); }
    static __device__ __forceinline__ unsigned long long bits(double x) {
        return (unsigned long long)__double_as_longlong(x);
    }
};
template <>
struct Staged<float> {
    static constexpr unsigned kSentinel = 0x7F8DEAD5u;
    static __device__ __forceinline__ unsigned ld(const float* p) {
        unsigned v;
        asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
        return v;
    }
    static __device__ __forceinline__ void st(float* p, unsigned v) {
        asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
    }
    static __device__ __forceinline__ float val(unsigned v) { return __uint_as_float(v); }
    static __device__ __forceinline__ unsigned bits(float x) { return __float_as_uint(x); }
};

template <typename T>
__device__ __forceinline__ void stage_put(T* p, T x) {
    Staged<T>::st(p, Staged<T>::bits(x));
}
template <typename T>
__device__ __forceinline__ void stage_clear(T* p) {
    Staged<T>::st(p, Staged<T>::kSentinel);
}
// Poll up to U elements p[u] (those with want[u]) until each holds a value;
// the loads of one round are all issued before any is tested.  Bounded:
// false after `limit` rounds, or once *status is non-zero (checked every
// 64 rounds); missing values then read as NaN.
template <typename T, int U>
__device__ __forceinline__ bool stage_take(const T* const (&p)[U], const bool (&want)[U], T (&out)[U],
                                           long long limit, const int32_t* status) {
    bool have[U];
#pragma unroll
    for (int u = 0; u < U; ++u) have[u] = !want[u];
    for (long long i = 0; i < limit; ++i) {
        decltype(Staged<T>::ld(p[0])) raw[U];
#pragma unroll
        for (int u = 0; u < U; ++u) raw[u] = have[u] ? Staged<T>::kSentinel : Staged<T>::ld(p[u]);
        bool all = true;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (!have[u] && raw[u] != Staged<T>::kSentinel) {
                out[u] = Staged<T>::val(raw[u]);
                have[u] = true;
            }
            all = all && have[u];
        }
        if (all) return true;
        if ((i & 63) == 63 && status != nullptr && *(const volatile int32_t*)status != 0) break;
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
        if (!have[u]) out[u] = T(NAN);
    return false;
}

// Unit-lower inverse Z = M^{-1} from its 8 x 8 diagonal blocks (already in
// z) by recursive doubling, 8 -> 16 -> 32: Z21 = -Z22 (M21 Z11).  M's strict
// lower part is in m (unit diagonal implied), u is scratch.
template <typename T>
__device__ void unit_inverse_doubling(T (*m)[kTile + 1], T (*z)[kTile + 1], T (*u)[kTile + 1]) {
    const int tid = threadIdx.x;
#pragma unroll 1
    for (int h = 8; h < kTile; h *= 2) {
        const int nout = (kTile / (2 * h)) * h * h;  // 128, then 256
        int r = 0, c = 0, o = 0;
        const bool act = tid < nout;
        if (act) {
            const int bi = tid / (h * h), rem = tid % (h * h);
            r = rem / h;
            c = rem % h;
            o = bi * 2 * h;
            // u = M21 Z11, Z11 unit lower: k >= c, Z11(c, c) = 1
            const T* mr = &m[o + h + r][o];
            T a0 = mr[c], a1 = T(0), a2 = T(0), a3 = T(0);
            int k = c + 1;
            for (; k + 3 < h; k += 4) {
                a0 = fma(mr[k], z[o + k][o + c], a0);
                a1 = fma(mr[k + 1], z[o + k + 1][o + c], a1);
                a2 = fma(mr[k + 2], z[o + k + 2][o + c], a2);
                a3 = fma(mr[k + 3], z[o + k + 3][o + c], a3);
            }
            for (; k < h; ++k) a0 = fma(mr[k], z[o + k][o + c], a0);
            u[o + h + r][o + c] = (a0 + a1) + (a2 + a3);
        }
        __syncthreads();
        if (act) {
            // Z21 = -Z22 u, Z22 unit lower: k <= r, Z22(r, r) = 1
            const T* zr = &z[o + h + r][o + h];
            T a0 = u[o + h + r][o + c], a1 = T(0), a2 = T(0), a3 = T(0);
            int k = 0;
            for (; k + 3 < r; k += 4) {
                a0 = fma(zr[k], u[o + h + k][o + c], a0);
                a1 = fma(zr[k + 1], u[o + h + k + 1][o + c], a1);
                a2 = fma(zr[k + 2], u[o + h + k + 2][o + c], a2);
                a3 = fma(zr[k + 3], u[o + h + k + 3][o + c], a3);
            }
            for (; k < r; ++k) a0 = fma(zr[k], u[o + h + k][o + c], a0);
            z[o + h + r][o + c] = -((a0 + a1) + (a2 + a3));
        }
        __syncthreads();
    }
}

// Cholesky + inverse of the diagonal tile at `tile` (nb <= 32), by one CTA,
// as L = M D^{1/2} (M unit lower, D the pivots) so that the sequential
// chain carries no square root:
//
// * the pivot warp (warp 0) produces column j: it applies the update of
//   column j-1 (held in its registers), reads the pivot d_j, forms 1/d_j
//   and M(:, j) = a'(:, j) / d_j, and publishes both (named barrier READY);
//   per column that is five FP64 instructions on its SM quarter, which no
//   other warp shares (warp 4 stays idle);
// * six worker warps (quarters 1-3) follow one column behind: with column
//   k they apply the rank-1 update to columns k+2.. (the pivot warp does
//   column k+1 itself), one triangle element per thread from a packed
//   index table, and advance the inverse of M's 8 x 8 diagonal blocks by
//   one row (Z(k, :) = -acc(k, :), acc(i, :) += M(i, k) Z(k, :) for i > k
//   in k's block), then signal UPD; the pivot warp waits for UPD(j-2)
//   before column j;
// * READY and UPD alternate between two barrier ids each, so neither side
//   can run two generations ahead of the other;
// * afterwards recursive doubling completes Z = M^{-1}, and
//   L = a' diag(d)^{-1/2}, L^{-1} = diag(d)^{-1/2} Z.
template <typename T>
__device__ void factor_tile(Smem<T>& S, T* tile, int64_t ld, int nb, int zero_right, T* tinv, int32_t* info,
                            int64_t row0) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int kPipe = 32 + 192;  // pivot warp + worker warps
    for (int e = tid; e < kTile * kTile; e += kTileThreads) {
        const int r = e / kTile, c = e % kTile;
        T v = T(0);
        if (r < nb && c <= r) v = __ldcg(tile + (int64_t)r * ld + c);
        else if (r >= nb && r == c) v = T(1);
        S.s[r][c] = v;
        S.tmp[r][c] = T(0);  // inverse accumulators
        S.x[r][c] = T(0);
        if (c <= r) S.tri[r * (r + 1) / 2 + c] = (unsigned short)((r << 8) | c);
    }
    if (tid == 0) S.fail = 0;
    __syncthreads();
    if (warp == 0) {
        T prev_a = T(0), prev_m = T(0);
        for (int j = 0; j < nb; ++j) {
            if (j >= 2) nbar_sync(3 + (j & 1), kPipe);  // UPD(j-2)
            T col = S.s[lane][j];
            if (j >= 1) col = fma(-prev_a, __shfl_sync(0xffffffffu, prev_m, j), col);
            const T d = __shfl_sync(0xffffffffu, col, j);
            const bool ok = pivot_ok(d);
            const T inv = ok ? rcp_pivot(d) : T(NAN);
            const T mcol = col * inv;
            if (lane >= j) S.s[lane][j] = col;
            if (lane > j) S.x[lane][j] = mcol;
            if (lane == j) {
                S.yv[j] = d;
                if (!ok && S.fail == 0) S.fail = j + 1;
            }
            nbar_arrive(1 + (j & 1), kPipe);  // READY(j)
            prev_a = col;
            prev_m = mcol;
        }
    } else if (warp != 4) {
        const int wid = (warp < 4 ? warp - 1 : warp - 2) * 32 + lane;  // 0..191
        for (int k = 0; k < nb; ++k) {
            nbar_sync(1 + (k & 1), kPipe);  // READY(k)
            const int w = nb - k - 2;
            const int n1 = w > 0 ? w * (w + 1) / 2 : 0;
            const int kb = k & ~7, kl = k - kb;
            const int ibe = (kb + 8 < nb ? kb + 8 : nb);  // end of k's 8-block
            const int n2 = (ibe - k - 1) * (kl + 1);
            for (int e = wid; e < n1 + n2; e += 192) {
                if (e < n1) {  // trailing rank-1 update of columns k+2..
                    const int rc = S.tri[e];
                    const int r = k + 2 + (rc >> 8), c = k + 2 + (rc & 0xff);
                    S.s[r][c] = fma(-S.s[r][k], S.x[c][k], S.s[r][c]);
                } else {  // inverse of k's 8-block: acc(i, c) += M(i, k) Z(k, c)
                    const int f = e - n1;
                    const int i = k + 1 + f / (kl + 1), c = kb + f % (kl + 1);
                    const T zk = (c == k) ? T(1) : -S.tmp[k][c];
                    S.tmp[i][c] = fma(S.x[i][k], zk, S.tmp[i][c]);
                }
            }
            if (k + 2 < nb) nbar_arrive(3 + (k & 1), kPipe);  // UPD(k)
        }
    }
    __syncthreads();
    for (int e = tid; e < kTile * kTile; e += kTileThreads) {  // Z's 8-blocks from the accumulators
        const int r = e / kTile, c = e % kTile;
        S.tmp[r][c] = (r == c) ? T(1) : -S.tmp[r][c];
    }
    if (tid < kTile) {
        const T d = S.yv[tid];
        S.yv[tid] = (tid < nb) ? rsq<T>(d) : T(1);
        S.u[tid][tid] = (tid < nb) ? d : T(1);  // pivot, read back below
    }
    __syncthreads();
    unit_inverse_doubling<T>(S.x, S.tmp, S.u);  // leaves the diagonal of u alone
    if (tid == 0 && S.fail != 0 && info != nullptr) atomicCAS(info, 0, (int32_t)(row0 + S.fail));
    for (int e = tid; e < kTile * kTile; e += kTileThreads) {
        const int r = e / kTile, c = e % kTile;
        T lv = T(0), xv = T(0);
        if (c < r) {
            lv = S.s[r][c] * S.yv[c];
            xv = S.tmp[r][c] * S.yv[r];
        } else if (c == r) {
            lv = S.u[r][r] * S.yv[r];
            xv = S.yv[r];
        }
        if (r < nb && c < nb) {
            tile[(int64_t)r * ld + c] = lv;
            tinv[r * kTile + c] = xv;
        }
        S.s[r][c] = lv;
        S.x[r][c] = xv;
    }
    for (int e = tid; e < nb * zero_right; e += kTileThreads) {
        const int r = e / zero_right, c = e % zero_right;
        tile[(int64_t)r * ld + nb + c] = T(0);
    }
    __syncthreads();
}

// The pipeline part of factor_tile alone, for the persistent column-block
// kernel: after it, S.x holds the strict lower part of M (zero elsewhere)
// and S.yv the pivots d (1 beyond nb), so L = M diag(d)^{1/2}; no inverse,
// no output.  The sequential chain is split between two warps on different
// SM quarters so that each carries as few FP64 instructions as possible:
//
// * warp 0 (pivot) keeps only the pivots: from 1/d_j and the pair
//   (q_{j+1}, e_{j+1}) = (a'_{j+1,j}^2, diagonal of column j+1 through
//   column j-1) it forms d_{j+1} = e_{j+1} - q_{j+1} / d_j with one FMA, tests
//   it and takes its reciprocal (three FMAs after an FP32 seed): four FP64
//   instructions per column;
// * warp 1 (companion) keeps column j of a' in registers: with 1/d_j it
//   forms M(:, j), publishes the column (READY), updates column j+1 with
//   column j and the diagonal with column j (registers), and hands the
//   pivot warp (q_{j+2}, e_{j+2}) -- four FP64 instructions per column;
// * warps 2, 3, 6, 7 (quarters 2 and 3) apply column k to the strict lower
//   part of columns k+2.. (the companion keeps the diagonal), then UPD;
// * with `mt` set, warp 4 publishes the factor outside the pipeline: the
//   companion counts its finished columns in S.pub (release at CTA scope);
//   the publisher takes every column finished since its last pass --
//   column k of M to mt[k][0..31] (transposed, so a column is one coalesced
//   row), d_k to dv[k] and d_k^{-1/2} to rv[k] -- makes them visible at GPU
//   scope and sets *colcount = col_base + (columns published), so other
//   CTAs consume the columns as they appear.  Its GPU-scope fences never
//   hold up the pivot pipeline; the chunks grow when a fence is slow.
//
// With `staged` the tile's lower part comes from that 32 x 32 staging
// buffer (ld 32) instead of `tile`, each element taken as its producer
// stores it and reset to the sentinel; `clear` (32 x 32) is reset to the
// sentinel; a poll that gives up (after `spin` rounds) sets *status =
// SGB_ERR_TIMEOUT.  With
// `vcols` warp 5 also hands the factor on by value, without fences: d_k to
// vcols[1024 + k] and column k of M to vcols[32 k .. 32 k + 31] as the
// companion finishes them; `vclear` (32 x 32 + 32) is reset first.
//
// Pivot <-> companion hand-offs use named barriers PQ (ids 5, 6) and QP
// (7, 8), READY/UPD ids 1-4 (companion + workers); every pair alternates
// between two ids so that no side can run two generations ahead (the
// arrival sequence was checked on a CPU model for nb = 1..32).
template <typename T>
__device__ void factor_tile_m(Smem<T>& S, const T* tile, int64_t ld, int nb, int32_t* info, int64_t row0,
                              T* mt = nullptr, T* dv = nullptr, T* rv = nullptr, unsigned* colcount = nullptr,
                              unsigned col_base = 0, T* staged = nullptr, T* clear = nullptr,
                              int32_t* status = nullptr, T* vcols = nullptr, T* vclear = nullptr,
                              long long spin = 1ll << 22) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int kCons = 32 * 5;  // companion + four workers
    constexpr int kPair = 64;
    T* iv = &S.tmp[0][0];  // 1/d_j
    T* qv = &S.tmp[1][0];  // a'_{j,j-1}^2
    T* ev = &S.tmp[2][0];  // diagonal of column j through column j-2
    constexpr int U = kTile * kTile / kTileThreads;
    bool timed_out = false;
    T sv[U];
    if (staged != nullptr) {  // lower part of the tile as its producers store it
        const T* sp[U];
        bool want[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int e = tid + u * kTileThreads, r = e / kTile, c = e % kTile;
            sp[u] = staged + e;
            want[u] = r < nb && c <= r;
        }
        timed_out = !stage_take<T, U>(sp, want, sv, spin, status);
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (want[u]) stage_clear(staged + tid + u * kTileThreads);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int e = tid + u * kTileThreads, r = e / kTile, c = e % kTile;
        T v = T(0);
        if (r < nb && c <= r) v = staged != nullptr ? sv[u] : __ldcg(tile + (int64_t)r * ld + c);
        else if (r >= nb && r == c) v = T(1);
        S.s[r][c] = v;
        S.x[r][c] = T(0);
        if (c < r) S.tri[r * (r - 1) / 2 + c] = (unsigned short)((r << 8) | c);  // strict lower, row-major
    }
    if (tid < kTile) S.yv[tid] = T(1);
    if (tid == 0) {
        S.fail = 0;
        S.pub = 0;
    }
    if (timed_out && status != nullptr) atomicExch(status, SGB_ERR_TIMEOUT);
    __syncthreads();
    if (warp == 0) {
        T d = S.s[0][0];
        bool ok = pivot_ok(d);
        T inv = ok ? rcp_pivot(d) : T(NAN);
        if (lane == 0 && !ok) S.fail = 1;
        for (int j = 0; j < nb; ++j) {
            if (lane == 0) {
                S.yv[j] = d;
                iv[j] = inv;
            }
            nbar_arrive(5 + (j & 1), kPair);  // PQ(j)
            if (j + 1 < nb) {
                nbar_sync(7 + ((j - 1) & 1), kPair);  // QP(j-1): q_{j+1}, e_{j+1}
                d = fma(-qv[j + 1], inv, ev[j + 1]);
                ok = pivot_ok(d);
                inv = ok ? rcp_pivot(d) : T(NAN);
                if (lane == 0 && !ok && S.fail == 0) S.fail = j + 2;
            }
        }
    } else if (warp == 1) {
        T col = S.s[lane][0];
        T diag = S.s[lane][lane];
        if (nb >= 2) {
            if (lane == 1) {
                qv[1] = col * col;
                ev[1] = diag;
            }
            nbar_arrive(8, kPair);  // QP(-1)
        }
        for (int j = 0; j < nb; ++j) {
            nbar_sync(5 + (j & 1), kPair);  // PQ(j)
            const T inv = iv[j];
            const T mcol = col * inv;
            if (lane >= j) S.s[lane][j] = col;
            if (lane > j) S.x[lane][j] = mcol;
            if (mt != nullptr) {  // column j (and d_j, seen through PQ(j)) to the publisher
                __syncwarp();
                if (lane == 0) asm volatile("st.release.cta.shared.u32 [%0], %1;" ::"r"(smem_u32(&S.pub)), "r"(j + 1)
                                            : "memory");
            }
            nbar_arrive(1 + (j & 1), kCons);  // READY(j)
            if (j >= 1) nbar_sync(3 + ((j - 1) & 1), kCons);  // UPD(j-1)
            if (j + 1 < nb) {
                const T mj1 = __shfl_sync(0xffffffffu, mcol, j + 1);
                const T col1 = fma(-col, mj1, S.s[lane][j + 1]);  // column j+1 through column j
                diag = fma(-col, mcol, diag);                      // diagonal through column j
                if (j + 2 < nb) {
                    if (lane == j + 2) {
                        qv[j + 2] = col1 * col1;
                        ev[j + 2] = diag;
                    }
                    nbar_arrive(7 + (j & 1), kPair);  // QP(j)
                }
                col = col1;
            }
        }
    } else if (warp == 4) {
        if (mt != nullptr) {
            int done = 0;
            long long spins = 0;
            while (done < nb) {
                int avail = 0;
                for (;;) {  // bounded: the companion finishes every column in any case
                    asm volatile("ld.acquire.cta.shared.u32 %0, [%1];" : "=r"(avail) : "r"(smem_u32(&S.pub)) : "memory");
                    if (avail > done || ++spins > (1ll << 26)) break;
                }
                if (avail <= done) break;  // the waits of the consumers time out and report it
                for (int k = done; k < avail; ++k) mt[k * kTile + lane] = S.x[lane][k];
                if (lane >= done && lane < avail) {
                    const T d = S.yv[lane];
                    dv[lane] = d;
                    rv[lane] = rsq<T>(d);
                }
                __threadfence();
                __syncwarp();
                if (lane == 0) atomicExch(colcount, col_base + (unsigned)avail);
                done = avail;
            }
        }
    } else if (warp == 5) {
        // every consumer of `clear` and `vclear` is done with them (they all
        // produced the staged values taken above)
        if (clear != nullptr)
            for (int e = lane; e < kTile * kTile; e += 32) stage_clear(clear + e);
        if (vclear != nullptr)
            for (int e = lane; e < kTile * kTile + kTile; e += 32) stage_clear(vclear + e);
        if (vcols != nullptr) {
            // the columns by value as the companion finishes them: d_k to
            // vcols[1024 + k], then column k of M to vcols[k * 32 + 0..31]
            int done = 0;
            long long spins = 0;
            while (done < nb) {
                int avail = 0;
                for (;;) {
                    asm volatile("ld.acquire.cta.shared.u32 %0, [%1];" : "=r"(avail) : "r"(smem_u32(&S.pub)) : "memory");
                    if (avail > done || ++spins > (1ll << 26)) break;
                }
                if (avail <= done) break;
                if (lane >= done && lane < avail) stage_put(vcols + kTile * kTile + lane, S.yv[lane]);
                for (int k = done; k < avail; ++k) stage_put(vcols + k * kTile + lane, S.x[lane][k]);
                done = avail;
            }
        }
    } else {
        const int wid = (warp < 4 ? warp - 2 : warp - 4) * 32 + lane;  // 0..127
        for (int k = 0; k < nb; ++k) {
            nbar_sync(1 + (k & 1), kCons);  // READY(k)
            const int w = nb - k - 2;
            const int n1 = w > 1 ? w * (w - 1) / 2 : 0;
            for (int e = wid; e < n1; e += 128) {  // column k on the strict lower part of columns k+2..
                const int rc = S.tri[e];
                const int r = k + 2 + (rc >> 8), c = k + 2 + (rc & 0xff);
                S.s[r][c] = fma(-S.s[r][k], S.x[c][k], S.s[r][c]);
            }
            if (k + 1 < nb) nbar_arrive(3 + (k & 1), kCons);  // UPD(k)
        }
    }
    __syncthreads();
    if (tid == 0 && S.fail != 0 && info != nullptr) atomicCAS(info, 0, (int32_t)(row0 + S.fail));
}

// The tile's L = M diag(d)^{1/2} from M (strict lower, in m), the pivots d
// (in dv) and d^{-1/2} (in rv) into `tile`, the upper part and the
// zero_right columns to the right of the tile set to zero.
template <typename T>
__device__ void tile_l_from_m(T (*m)[kTile + 1], const T* dv, const T* rv, T* tile, int64_t ld, int nb,
                              int zero_right) {
    const int tid = threadIdx.x;
    for (int e = tid; e < nb * nb; e += kTileThreads) {
        const int r = e / nb, c = e - (e / nb) * nb;
        T lv = T(0);
        if (c <= r) {
            const T sq = dv[c] * rv[c];  // sqrt(d_c)
            lv = (c < r) ? m[r][c] * sq : sq;
        }
        tile[(int64_t)r * ld + c] = lv;
    }
    for (int e = tid; e < nb * zero_right; e += kTileThreads) {
        const int r = e / zero_right, c = e % zero_right;
        tile[(int64_t)r * ld + nb + c] = T(0);
    }
    __syncthreads();
}

}  // namespace sgb
