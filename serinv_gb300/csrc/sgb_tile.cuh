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
    T yv[kTile];
    int fail;
    int flag;
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

// A(p): Cholesky + inverse of the diagonal tile at `tile` (nb <= 32), by one CTA.
template <typename T>
__device__ void factor_tile(Smem<T>& S, T* tile, int64_t ld, int nb, int zero_right, T* tinv, int32_t* info,
                            int64_t row0) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int e = tid; e < kTile * kTile; e += kTileThreads) {
        const int r = e / kTile, c = e % kTile;
        T v = T(0);
        if (r < nb && c <= r) v = __ldcg(tile + (int64_t)r * ld + c);
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
            const bool bad = !pivot_ok(d);
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
    for (int e = tid; e < nb * nb; e += kTileThreads) {
        const int r = e / nb, c = e % nb;
        tile[(int64_t)r * ld + c] = (c <= r) ? S.s[r][c] : T(0);
        tinv[r * kTile + c] = S.x[r][c];
    }
    for (int e = tid; e < nb * zero_right; e += kTileThreads) {
        const int r = e / zero_right, c = e % zero_right;
        tile[(int64_t)r * ld + nb + c] = T(0);
    }
}


}  // namespace sgb
