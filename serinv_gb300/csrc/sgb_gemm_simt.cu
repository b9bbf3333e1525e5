// Grouped, batched SIMT GEMM in the storage precision (FP64 DFMA / FP32 FFMA).
//
// One launch processes up to kMaxProbs independent problems
//   Cout = alpha * sum_t op(A_t) op(B_t) + beta * op(Cin)
// each optionally batched.  Every CTA computes one 32 x 32 output tile.
// The tile is small on purpose: on GB300 the FP64 pipe retires about two
// DFMA per SM per clock, so a 32 x 32 x 512 tile already runs for ~100 us
// and small tiles are what spreads the block-step GEMMs (512 x 512) over
// all 152 SMs.  Operand tiles are staged through shared memory with
// coalesced loads for either storage orientation.
#include "sgb_internal.cuh"

namespace sgb {

namespace {

constexpr int BM = 32, BN = 32, BK = 16, NT = 256;
constexpr int TM = 2, TN = 2;  // rows ty + 16*i, cols tx + 16*j

template <typename T>
__device__ __forceinline__ void k_range(const GemmTerm<T>& t, int m0, int n0, int& klo, int& khi) {
    klo = 0;
    khi = t.K;
    switch (t.kmode) {
        case KM_GE_N0: klo = n0; break;
        case KM_LT_N1: khi = min(t.K, n0 + BN); break;
        case KM_GE_M0: klo = m0; break;
        case KM_LT_M1: khi = min(t.K, m0 + BM); break;
        default: break;
    }
}

template <typename T>
__global__ void __launch_bounds__(NT) k_gemm_simt(const __grid_constant__ GemmLaunch<T> L) {
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN + 1];

    const int tile = blockIdx.x;
    int pi = 0;
#pragma unroll 1
    for (int q = 1; q < L.np; ++q)
        if (tile >= L.p[q].tile_begin) pi = q;
    const GemmProb<T>& P = L.p[pi];

    int local = tile - P.tile_begin;
    const int per_inst = P.tiles_m * P.tiles_n;
    const int inst = local / per_inst;
    local -= inst * per_inst;
    const int tm = local / P.tiles_n;
    const int tn = local - tm * P.tiles_n;
    const int m0 = tm * BM, n0 = tn * BN;
    if (P.lower_only && n0 >= m0 + BM) return;  // strictly above the diagonal

    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;

    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

#pragma unroll 1
    for (int ti = 0; ti < P.nterms; ++ti) {
        const GemmTerm<T>& t = P.term[ti];
        const T* A = t.A + (int64_t)inst * t.strideA;
        const T* B = t.B + (int64_t)inst * t.strideB;
        int klo, khi;
        k_range(t, m0, n0, klo, khi);
#pragma unroll 1
        for (int k0 = klo; k0 < khi; k0 += BK) {
            // A tile: op(A)[m0 .. m0+BM) x [k0 .. k0+BK)
#pragma unroll
            for (int e = tid; e < BM * BK; e += NT) {
                int m, k;
                if (t.transA) { m = e % BM; k = e / BM; }
                else          { k = e % BK; m = e / BK; }
                const int gm = m0 + m, gk = k0 + k;
                T v = T(0);
                if (gm < P.M && gk < khi)
                    v = t.transA ? A[(int64_t)gk * t.lda + gm] : A[(int64_t)gm * t.lda + gk];
                As[k][m] = v;
            }
            // B tile: op(B)[k0 .. k0+BK) x [n0 .. n0+BN)
#pragma unroll
            for (int e = tid; e < BK * BN; e += NT) {
                int n, k;
                if (t.transB) { k = e % BK; n = e / BK; }
                else          { n = e % BN; k = e / BN; }
                const int gn = n0 + n, gk = k0 + k;
                T v = T(0);
                if (gn < P.N && gk < khi)
                    v = t.transB ? B[(int64_t)gn * t.ldb + gk] : B[(int64_t)gk * t.ldb + gn];
                Bs[k][n] = v;
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < BK; ++kk) {
                T a[TM], bb[TN];
#pragma unroll
                for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < TN; ++j) bb[j] = Bs[kk][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < TM; ++i)
#pragma unroll
                    for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
            }
            __syncthreads();
        }
    }

    T* C = P.Cout + (int64_t)inst * P.strideC;
    const T* Ci = P.Cin ? P.Cin + (int64_t)inst * P.strideCin : nullptr;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        const int gm = m0 + ty + 16 * i;
        if (gm >= P.M) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int gn = n0 + tx + 16 * j;
            if (gn >= P.N) continue;
            T v = P.alpha * acc[i][j];
            if (Ci != nullptr && P.beta != T(0)) {
                const T c = P.transCin ? Ci[(int64_t)gn * P.ldcin + gm] : Ci[(int64_t)gm * P.ldcin + gn];
                v = fma(P.beta, c, v);
            }
            C[(int64_t)gm * P.ldc + gn] = v;
        }
    }
}

// Skinny products (N <= 8: the solves' right-hand sides).  A 32 x 32 tile
// would run a K-long dependent FMA chain per output; here each CTA owns 8
// output rows and all N columns (so even a 256-row product spreads over 32
// SMs), and the K dimension is spread over the threads: for a row-major
// op(A) warp w takes row w and its lanes walk k (coalesced, warp-shuffle
// reduction); for a transposed op(A) a lane takes row lane % 8 and one of
// 32 interleaved k streams (8 consecutive rows are one 64-byte segment),
// reduced by shuffles within the warp and through shared memory across the
// eight warps.  B is staged 256 rows of k at a time.  Reduction orders are
// fixed, so results are reproducible.
constexpr int SK_ROWS = 8, SK_NMAX = 8, SK_KC = 256;

template <typename T>
__global__ void __launch_bounds__(NT) k_gemm_skinny(const __grid_constant__ GemmLaunch<T> L) {
    __shared__ T Bs[SK_KC][SK_NMAX];
    __shared__ T red[NT / 32][SK_ROWS][SK_NMAX];
    __shared__ T Cs[SK_ROWS][SK_NMAX + 1];

    const int tile = blockIdx.x;
    int pi = 0;
#pragma unroll 1
    for (int q = 1; q < L.np; ++q)
        if (tile >= L.p[q].tile_begin) pi = q;
    const GemmProb<T>& P = L.p[pi];
    const int local = tile - P.tile_begin;
    const int inst = local / P.tiles_m;
    const int m0 = (local - inst * P.tiles_m) * SK_ROWS;
    const int N = P.N;
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    for (int e = tid; e < SK_ROWS * (SK_NMAX + 1); e += NT) Cs[e / (SK_NMAX + 1)][e % (SK_NMAX + 1)] = T(0);

#pragma unroll 1
    for (int ti = 0; ti < P.nterms; ++ti) {
        const GemmTerm<T>& t = P.term[ti];
        const T* A = t.A + (int64_t)inst * t.strideA;
        const T* B = t.B + (int64_t)inst * t.strideB;
        int klo = 0, khi = t.K;
        switch (t.kmode) {
            case KM_GE_N0: break;
            case KM_LT_N1: khi = min(t.K, N); break;
            case KM_GE_M0: klo = m0; break;
            case KM_LT_M1: khi = min(t.K, m0 + SK_ROWS); break;
            default: break;
        }
#pragma unroll 1
        for (int kc0 = klo; kc0 < khi; kc0 += SK_KC) {
            const int kc1 = min(khi, kc0 + SK_KC);
            __syncthreads();
            for (int e = tid; e < (kc1 - kc0) * N; e += NT) {
                const int k = e / N, j = e - k * N;
                Bs[k][j] = B[(int64_t)(kc0 + k) * t.ldb + j];
            }
            __syncthreads();
            T acc[SK_NMAX];
#pragma unroll
            for (int j = 0; j < SK_NMAX; ++j) acc[j] = T(0);
            if (!t.transA) {
                const int gm = m0 + w;
                if (gm < P.M) {
                    const T* Ar = A + (int64_t)gm * t.lda;
                    for (int k = kc0 + lane; k < kc1; k += 32) {
                        const T a = Ar[k];
#pragma unroll
                        for (int j = 0; j < SK_NMAX; ++j)
                            if (j < N) acc[j] = fma(a, Bs[k - kc0][j], acc[j]);
                    }
                }
#pragma unroll
                for (int j = 0; j < SK_NMAX; ++j) {
                    if (j >= N) continue;
                    T v = acc[j];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                    if (lane == 0) Cs[w][j] += v;
                }
            } else {
                const int r = lane & 7, gm = m0 + r;
                if (gm < P.M)
                    for (int k = kc0 + w * 4 + (lane >> 3); k < kc1; k += 32) {
                        const T a = A[(int64_t)k * t.lda + gm];
#pragma unroll
                        for (int j = 0; j < SK_NMAX; ++j)
                            if (j < N) acc[j] = fma(a, Bs[k - kc0][j], acc[j]);
                    }
#pragma unroll
                for (int j = 0; j < SK_NMAX; ++j) {
                    T v = acc[j];
                    v += __shfl_xor_sync(0xffffffffu, v, 8);
                    v += __shfl_xor_sync(0xffffffffu, v, 16);
                    if (lane < 8) red[w][lane][j] = v;
                }
                __syncthreads();
                for (int e = tid; e < SK_ROWS * N; e += NT) {
                    const int rr = e / N, j = e - rr * N;
                    T v = T(0);
#pragma unroll
                    for (int q = 0; q < NT / 32; ++q) v += red[q][rr][j];
                    Cs[rr][j] += v;
                }
            }
        }
    }
    __syncthreads();
    T* C = P.Cout + (int64_t)inst * P.strideC;
    const T* Ci = P.Cin ? P.Cin + (int64_t)inst * P.strideCin : nullptr;
    for (int e = tid; e < SK_ROWS * N; e += NT) {
        const int r = e / N, j = e - r * N, gm = m0 + r;
        if (gm >= P.M) continue;
        T v = P.alpha * Cs[r][j];
        if (Ci != nullptr && P.beta != T(0)) {
            const T c = P.transCin ? Ci[(int64_t)j * P.ldcin + gm] : Ci[(int64_t)gm * P.ldcin + j];
            v = fma(P.beta, c, v);
        }
        C[(int64_t)gm * P.ldc + j] = v;
    }
}

// FP32 products with a 64 x 64 output tile per CTA (4 x 4 per thread,
// 16-byte shared-memory operand reads, the next K slab fetched into
// registers during the current slab's FMAs).  The FP32 pipe retires 128
// FFMA per SM per clock, 64 times the FP64 rate, so FP32 products are bound
// by operand traffic, not arithmetic: the 32 x 32 tile's one shared-memory
// read per FMA caps it far below the FFMA rate.  Same problem semantics as
// k_gemm_simt, including `lower_only` at its 32 x 32 granularity (an
// element is written unless its 32 x 32 tile lies strictly above the
// diagonal), so either kernel may serve a launch.
constexpr int WB = 64, WK = 16;

__global__ void __launch_bounds__(NT) k_gemm_wide(const __grid_constant__ GemmLaunch<float> L) {
    __shared__ __align__(16) float As[WK][WB + 4];
    __shared__ __align__(16) float Bs[WK][WB + 4];

    const int tile = blockIdx.x;
    int pi = 0;
#pragma unroll 1
    for (int q = 1; q < L.np; ++q)
        if (tile >= L.p[q].tile_begin) pi = q;
    const GemmProb<float>& P = L.p[pi];
    int local = tile - P.tile_begin;
    const int per_inst = P.tiles_m * P.tiles_n;
    const int inst = local / per_inst;
    local -= inst * per_inst;
    const int tm = local / P.tiles_n;
    const int tn = local - tm * P.tiles_n;
    const int m0 = tm * WB, n0 = tn * WB;
    if (P.lower_only && n0 >= m0 + WB) return;

    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;

#pragma unroll 1
    for (int ti = 0; ti < P.nterms; ++ti) {
        const GemmTerm<float>& t = P.term[ti];
        const float* A = t.A + (int64_t)inst * t.strideA;
        const float* B = t.B + (int64_t)inst * t.strideB;
        int klo = 0, khi = t.K;
        switch (t.kmode) {
            case KM_GE_N0: klo = n0; break;
            case KM_LT_N1: khi = min(t.K, n0 + WB); break;
            case KM_GE_M0: klo = m0; break;
            case KM_LT_M1: khi = min(t.K, m0 + WB); break;
            default: break;
        }
        // slab element e = tid + 256 q (q < 4): A as (m, k), B as (k, n),
        // with the index order that makes the global reads coalesced
        float ra[4], rb[4];
        auto fetch = [&](int k0) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = tid + NT * q;
                int m, k;
                if (t.transA) { m = e % WB; k = e / WB; }
                else          { k = e % WK; m = e / WK; }
                const int gm = m0 + m, gk = k0 + k;
                ra[q] = (gm < P.M && gk < khi)
                            ? (t.transA ? A[(int64_t)gk * t.lda + gm] : A[(int64_t)gm * t.lda + gk])
                            : 0.f;
                int n;
                if (t.transB) { k = e % WK; n = e / WK; }
                else          { n = e % WB; k = e / WB; }
                const int gn = n0 + n;
                const int gk2 = k0 + k;
                rb[q] = (gn < P.N && gk2 < khi)
                            ? (t.transB ? B[(int64_t)gn * t.ldb + gk2] : B[(int64_t)gk2 * t.ldb + gn])
                            : 0.f;
            }
        };
        auto park = [&]() {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = tid + NT * q;
                int m, k;
                if (t.transA) { m = e % WB; k = e / WB; }
                else          { k = e % WK; m = e / WK; }
                As[k][m] = ra[q];
                int n;
                if (t.transB) { k = e % WK; n = e / WK; }
                else          { n = e % WB; k = e / WB; }
                Bs[k][n] = rb[q];
            }
        };
        if (klo < khi) fetch(klo);
#pragma unroll 1
        for (int k0 = klo; k0 < khi; k0 += WK) {
            __syncthreads();  // the previous slab's reads are done
            park();
            __syncthreads();
            if (k0 + WK < khi) fetch(k0 + WK);
#pragma unroll
            for (int kk = 0; kk < WK; ++kk) {
                const float4 a = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
                const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
                const float av[4] = {a.x, a.y, a.z, a.w};
                const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
            }
        }
        __syncthreads();
    }

    float* C = P.Cout + (int64_t)inst * P.strideC;
    const float* Ci = P.Cin ? P.Cin + (int64_t)inst * P.strideCin : nullptr;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int gm = m0 + ty * 4 + i;
        if (gm >= P.M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gn = n0 + tx * 4 + j;
            if (gn >= P.N) continue;
            if (P.lower_only && (gn >> 5) > (gm >> 5)) continue;
            float v = P.alpha * acc[i][j];
            if (Ci != nullptr && P.beta != 0.f) {
                const float c = P.transCin ? Ci[(int64_t)gn * P.ldcin + gm] : Ci[(int64_t)gm * P.ldcin + gn];
                v = fmaf(P.beta, c, v);
            }
            C[(int64_t)gm * P.ldc + gn] = v;
        }
    }
}

inline void launch_wide(const GemmLaunch<float>& L, unsigned grid, cudaStream_t s) {
    k_gemm_wide<<<grid, NT, 0, s>>>(L);
}
inline void launch_wide(const GemmLaunch<double>&, unsigned, cudaStream_t) {}  // never selected

// The wide kernel serves an FP32 launch when one of its problems has a
// 64 x 64 output tile's worth of rows and columns (smaller problems of the
// same launch ride along in partly empty tiles).
template <typename T>
bool wide_ok(const GemmProb<T>* probs, int np) {
    if (sizeof(T) != 4) return false;
    for (int i = 0; i < np; ++i)
        if (probs[i].batch > 0 && probs[i].M >= WB && probs[i].N >= WB) return true;
    return false;
}

// Bytes an operand of `rows` x `cols` (leading dimension ld) spans over the
// batch, as [lo, hi).
template <typename T>
void span(const T* p, int64_t rows, int64_t cols, int64_t ld, int64_t stride, int32_t batch, uintptr_t& lo,
          uintptr_t& hi) {
    lo = (uintptr_t)p;
    hi = lo + (uintptr_t)(((rows - 1) * ld + cols + (int64_t)(batch - 1) * stride) * (int64_t)sizeof(T));
}

// The skinny kernel serves a launch when every problem has N <= 8, no
// transposed B, no lower-only restriction, and no operand overlapping its
// output (each CTA reads all of B while others write their rows of C).
template <typename T>
bool skinny_ok(const GemmProb<T>* probs, int np) {
    bool any = false;
    for (int i = 0; i < np; ++i) {
        const GemmProb<T>& p = probs[i];
        if (p.M <= 0 || p.N <= 0 || p.batch <= 0) continue;
        if (p.N > SK_NMAX || p.lower_only) return false;
        any = true;
        uintptr_t clo, chi;
        span(p.Cout, p.M, p.N, p.ldc, p.strideC, p.batch, clo, chi);
        for (int t = 0; t < p.nterms; ++t) {
            const GemmTerm<T>& g = p.term[t];
            if (g.transB) return false;
            uintptr_t lo, hi;
            span(g.B, g.K, p.N, g.ldb, g.strideB, p.batch, lo, hi);
            if (lo < chi && clo < hi) return false;
            if (g.transA) span(g.A, g.K, p.M, g.lda, g.strideA, p.batch, lo, hi);
            else span(g.A, p.M, g.K, g.lda, g.strideA, p.batch, lo, hi);
            if (lo < chi && clo < hi) return false;
        }
    }
    return any;
}

}  // namespace

template <typename T>
double useful_flops(const GemmProb<T>& p) {
    // 2 * sum over output elements of the K-range each term needs.
    double f = 0.0;
    for (int t = 0; t < p.nterms; ++t) {
        const GemmTerm<T>& tm = p.term[t];
        const int64_t K = tm.K;
        double s = 0.0;
        if (tm.kmode == KM_GE_M0 || tm.kmode == KM_LT_M1) {
            for (int64_t m = 0; m < p.M; ++m) {
                const int64_t kl = tm.kmode == KM_GE_M0 ? (K - m > 0 ? K - m : 0) : (m + 1 < K ? m + 1 : K);
                const int64_t ncols = p.lower_only ? (m + 1 < p.N ? m + 1 : p.N) : p.N;
                s += (double)kl * ncols;
            }
        } else {
            for (int64_t n = 0; n < p.N; ++n) {
                int64_t kl = K;
                if (tm.kmode == KM_GE_N0) kl = K - n > 0 ? K - n : 0;
                if (tm.kmode == KM_LT_N1) kl = n + 1 < K ? n + 1 : K;
                const int64_t nrows = p.lower_only ? (p.M - n > 0 ? p.M - n : 0) : p.M;
                s += (double)kl * nrows;
            }
        }
        f += 2.0 * s;
    }
    return f * p.batch;
}

template double useful_flops<double>(const GemmProb<double>&);
template double useful_flops<float>(const GemmProb<float>&);

template <typename T>
cudaError_t gemm_simt(GemmProb<T>* probs, int np, cudaStream_t s) {
    GemmLaunch<T> L;
    L.np = 0;
    int64_t total = 0;
    const bool skinny = skinny_ok<T>(probs, np);
    const bool wide = !skinny && wide_ok<T>(probs, np);
    const int tile_m = skinny ? SK_ROWS : (wide ? WB : BM);
    for (int i = 0; i < np; ++i) {
        GemmProb<T> p = probs[i];
        if (p.M <= 0 || p.N <= 0 || p.batch <= 0) continue;
        p.tiles_m = (int32_t)ceil_div(p.M, tile_m);
        p.tiles_n = skinny ? 1 : (int32_t)ceil_div(p.N, wide ? WB : BN);
        p.tile_begin = (int32_t)total;
        total += (int64_t)p.tiles_m * p.tiles_n * p.batch;
        L.p[L.np++] = p;
        if (L.np == kMaxProbs && i + 1 < np) return cudaErrorInvalidValue;
    }
    if (L.np == 0) return cudaSuccess;
    if (total > 0x7fffffff) return cudaErrorInvalidValue;
    L.total_tiles = (int32_t)total;
    double fl = 0.0;
    for (int i = 0; i < L.np; ++i) fl += useful_flops<T>(L.p[i]);
    prof_before(s, SGB_KCLASS_GEMM);
    if (skinny) k_gemm_skinny<T><<<(unsigned)total, NT, 0, s>>>(L);
    else if (wide) launch_wide(L, (unsigned)total, s);
    else k_gemm_simt<T><<<(unsigned)total, NT, 0, s>>>(L);
    prof_after(SGB_KCLASS_GEMM, s, fl);
    return cudaGetLastError();
}

template cudaError_t gemm_simt<double>(GemmProb<double>*, int, cudaStream_t);
template cudaError_t gemm_simt<float>(GemmProb<float>*, int, cudaStream_t);

}  // namespace sgb
