// Tensor-core (tcgen05) FP64-storage GEMM built from exact bf16 slice products.
//
// Each FP64 operand row (rows of op(A), columns of op(B)) is scaled by a
// power of two 2^e so its entries lie in (-1, 1), turned into a signed
// fixed-point integer X = round(x * 2^(7S)), and cut into S balanced base-128
// digits d_0 .. d_{S-1} (|d_0| <= 128, |d_p| <= 64).  Slice p stores
// w_p = d_p * 2^(-7p) in bf16 (exact: at most 8 significant bits).  Then
//
//   C[m][n] = 2^(eA[m] + eB[n] - 14) * sum_{p+q <= S-1} (A_p B_q)[m][n]
//
// The products are exact in the FP32 accumulator; grouping them by level
// l = p + q keeps every partial sum of a level an integer multiple of
// 2^(-7l) whose magnitude stays below 2^24 of those units: per k a level-l
// term is at most 2^14 + (l-1) 2^12 units, so levels 0..4 are exact for
// K <= kTcMaxK = 576.  Each level up to 4 has its own TMEM accumulator; for
// S = 7 the last accumulator also takes levels 5 and 6 (weight <= 2^-35).
// The truncation error of S digits is 2^-(7S+1) of the row maximum.  The
// epilogue adds the accumulators exactly as an FP32 pair (two-sum), widens
// the pair with integer bit operations, adds it in FP64 (one FP64 add),
// applies the power-of-two scale on the exponent bits and alpha/beta, and
// stores FP64: two FP64 instructions per element, because every FP64 warp
// instruction occupies its SM quarter for ~64 cycles on this part.
//
// This is the published Ozaki error-free splitting idea (Ozaki, Ogita,
// Oishi, Rump) specialised to fixed-point digits and level-grouped exact
// tensor-core accumulation.
//
// Kernel structure (one CTA = one 128 x BN output tile, 6 warps):
//   * the split kernel writes every slice pre-tiled: one contiguous chunk per
//     (row tile, 32-wide K block) already in the no-swizzle K-major
//     core-matrix order (8 rows x 16 bytes per core matrix) that the MMA
//     descriptors read, so each stage is 2S plain bulk copies;
//   * warp 4 (producer) streams the chunks with cp.async.bulk into a ring of
//     2-4 stages, each guarded by a full/empty mbarrier pair;
//   * warp 5 issues tcgen05.mma (cta_group::1, kind::f16, bf16 inputs, FP32
//     accumulation in TMEM) and tcgen05.commit, which frees a stage when its
//     MMAs have read it;
//   * warps 0-3 wait for the last commit, read their 32 TMEM lanes with
//     tcgen05.ld and write FP64;
//   * every mbarrier wait is bounded; on timeout an error word is set and
//     the kernel drains (bounded) and frees its TMEM before returning.
#include <cuda_bf16.h>
#include <string.h>

#include <mutex>

#include "sgb_internal.cuh"

namespace sgb {

namespace {

constexpr int TC_BM = 128;
constexpr int TC_BK = 32;
constexpr int kMaxTcProbs = 4;
#ifndef SGB_TC_SM_COUNT
#define SGB_TC_SM_COUNT 148
#endif
#ifndef SGB_TC_MAX_SPLIT
#define SGB_TC_MAX_SPLIT 4
#endif
constexpr int64_t kTcSmCount = SGB_TC_SM_COUNT;  // CTAs one launch should keep busy (152 SMs)
constexpr int kTcMaxSplit = SGB_TC_MAX_SPLIT;    // CTAs per cluster of a K-split tile (<= 8)
constexpr int kMaxSplitJobs = 2 * kMaxTcProbs;  // probs x operands
constexpr long long kSpinLimit = 1ll << 22;         // bounded drain waits after an error (~1 s)

// ---------------------------------------------------------------- split

struct SplitSrc {
    const double* X;
    int64_t ld_r, ld_k;   // element (r, k) at X[r*ld_r + k*ld_k]
    int64_t stride;       // batch stride (elements)
    int32_t K, koff;      // source K extent; destination K offset (multiple of TC_BK)
};

// One operand of one problem: the rows of op(A) (or the columns of op(B))
// over the K ranges of all its terms.
struct SplitJob {
    SplitSrc src[2];
    int32_t nsrc;
    __nv_bfloat16* out;   // per instance: [S][Rpad/RT][Kpad/32] chunks of RT x 32 (core-matrix order)
    int32_t* exps;        // [Rpad] per instance (biased FP64 exponent of the row max, 0 for a zero row)
    int64_t out_stride, exp_stride;
    int32_t R, Rpad, Kpad;
    int32_t RT;           // rows per chunk: 128 for A, the tile width for B
    int32_t batch;
    int32_t strips, strip_begin;  // kSplitRows-row strips per instance; first CTA of the job
};

constexpr int kSplitRows = 8;
constexpr int kSplitThreads = 512;  // two CTAs per SM, eight warps per scheduler: latency bound
constexpr int kSplitLd = kTcMaxK + 1;  // odd stride: conflict-free row and column access

struct SplitLaunch {
    SplitJob j[kMaxSplitJobs];
    int32_t nj;
    int32_t S;
};

__device__ __forceinline__ int find_job(const SplitLaunch& L, int cta) {
    int ji = 0;
#pragma unroll 1
    for (int q = 1; q < L.nj; ++q)
        if (cta >= L.j[q].strip_begin) ji = q;
    return ji;
}

// Balanced base-128 digits of x scaled by the row exponent Erow (biased).
template <int S>
__device__ __forceinline__ void digits(double x, int Erow, int (&d)[S]) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int Ex = (int)((bits >> 52) & 0x7ff);
#pragma unroll
    for (int p = 0; p < S; ++p) d[p] = 0;
    if (Ex == 0 || Erow == 0) return;  // zero, subnormal (flushed) or zero row
    const long long m = (long long)((bits & ((1ull << 52) - 1)) | (1ull << 52));
    const int rs = Erow - Ex + 53 - 7 * S;  // right shift; >= 53 - 7S > 0 for S <= 7
    long long X;
    if (rs >= 62) X = 0;
    else if (rs <= 0) X = m << (-rs);
    else X = (m + (1ll << (rs - 1))) >> rs;
    if (bits >> 63) X = -X;
    // |X| < 2^(7S+1) <= 2^50: the low L digits come out of the low 7L bits
    // and the rest out of the high part, all in 32-bit arithmetic (the
    // balanced digit v = ((x mod 128) ^ 64) - 64 lies in [-64, 63]; removing
    // the low digits leaves a carry of 0 or 1 for the high part).
    constexpr int L = (S - 1) < 3 ? (S - 1) : 3;
    int lo = (int)(X & ((1ll << (7 * L)) - 1));
    int hi = (int)(X >> (7 * L));
#pragma unroll
    for (int p = S - 1; p >= S - L; --p) {
        const int v = ((lo & 127) ^ 64) - 64;
        d[p] = v;
        lo = (lo - v) >> 7;
    }
    hi += lo;
#pragma unroll
    for (int p = S - L - 1; p >= 1; --p) {
        const int v = ((hi & 127) ^ 64) - 64;
        d[p] = v;
        hi = (hi - v) >> 7;
    }
    d[0] = hi;
}

// Programmatic dependent launch: the kernels of a product are launched
// with programmatic stream serialization, so a launch may start while its
// predecessor in the stream drains.  Every kernel waits for the
// predecessor's completion (and memory) before its first global access,
// then lets its own successor start launching.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// One CTA per strip of kSplitRows rows of one operand instance: the whole
// strip (all terms, K <= kTcMaxK) is staged in shared memory with coalesced
// loads, each row's largest exponent is found by one warp, and the S slices
// of every element are written in the chunk layout the MMA descriptors
// read -- padding rows and the K padding of each term as zeros, so the
// buffers need no clearing beforehand.
template <int S>
__global__ void __launch_bounds__(kSplitThreads) k_split(const __grid_constant__ SplitLaunch L) {
    __shared__ double t[kSplitRows][kSplitLd];
    __shared__ int ex[kSplitRows];
    pdl_enter();
    const SplitJob& J = L.j[find_job(L, blockIdx.x)];
    const int local = blockIdx.x - J.strip_begin;
    const int inst = local / J.strips;
    const int r0 = (local - inst * J.strips) * kSplitRows;
    const int tid = threadIdx.x;
    // Each source covers [koff, koff + Kp) of the strip (Kp = K rounded up to
    // 32); elements past K or past the last row are written as zeros, so
    // every element of the strip is written once.  A thread issues all its
    // loads before it stores any (no index division: rows of a row-major
    // source are walked by consecutive threads, a transposed source by four
    // rows times 128 k per pass).
    for (int q = 0; q < J.nsrc; ++q) {
        const SplitSrc& src = J.src[q];
        const double* X = src.X + (int64_t)inst * src.stride;
        const int Kp = (src.K + TC_BK - 1) / TC_BK * TC_BK;
        if (src.ld_k == 1) {
            constexpr int KU = (kTcMaxK + kSplitThreads - 1) / kSplitThreads;  // 2
            double v[kSplitRows][KU];
#pragma unroll
            for (int rr = 0; rr < kSplitRows; ++rr)
#pragma unroll
                for (int u = 0; u < KU; ++u) {
                    const int k = tid + u * kSplitThreads, r = r0 + rr;
                    v[rr][u] = (k < src.K && r < J.R) ? __ldg(X + (int64_t)r * src.ld_r + k) : 0.0;
                }
#pragma unroll
            for (int rr = 0; rr < kSplitRows; ++rr)
#pragma unroll
                for (int u = 0; u < KU; ++u) {
                    const int k = tid + u * kSplitThreads;
                    if (k < Kp) t[rr][src.koff + k] = v[rr][u];
                }
        } else {
            constexpr int KS = kSplitThreads / kSplitRows;  // 64 k per pass
            constexpr int KU = (kTcMaxK + KS - 1) / KS;     // 9
            const int rr = tid % kSplitRows, r = r0 + rr;
            double v[KU];
#pragma unroll
            for (int u = 0; u < KU; ++u) {
                const int k = tid / kSplitRows + u * KS;
                v[u] = (k < src.K && r < J.R) ? __ldg(X + (int64_t)r * src.ld_r + (int64_t)k * src.ld_k) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < KU; ++u) {
                const int k = tid / kSplitRows + u * KS;
                if (k < Kp) t[rr][src.koff + k] = v[u];
            }
        }
    }
    if (J.nsrc == 0)
        for (int e = tid; e < kSplitRows * J.Kpad; e += kSplitThreads) t[e / J.Kpad][e % J.Kpad] = 0.0;
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    if (warp < kSplitRows) {
        int emax = 0;
        for (int k = lane; k < J.Kpad; k += 32) {
            const int e = (int)(((unsigned long long)__double_as_longlong(t[warp][k]) >> 52) & 0x7ff);
            emax = e > emax ? e : emax;
        }
        emax = __reduce_max_sync(0xffffffffu, emax);
        if (lane == 0) {
            ex[warp] = emax;
            J.exps[(int64_t)inst * J.exp_stride + r0 + warp] = emax;
        }
    }
    __syncthreads();
    __nv_bfloat16* out = J.out + (int64_t)inst * J.out_stride;
    const int64_t slice = (int64_t)J.Rpad * J.Kpad;
    const int nkb = J.Kpad / 32, RT = J.RT;
    // Eight consecutive k of one row are contiguous (16 bytes) in the core-
    // matrix order [k/8][row/8][row%8][k%8] of a chunk: a thread digits one
    // such group and writes each slice with a single 16-byte store.
    const float w7[7] = {1.0f, 0x1p-7f, 0x1p-14f, 0x1p-21f, 0x1p-28f, 0x1p-35f, 0x1p-42f};
    for (int g = tid; g < kSplitRows * (J.Kpad / 8); g += kSplitThreads) {
        const int rr = g % kSplitRows, k0 = (g / kSplitRows) * 8;
        const int r = r0 + rr;
        const int rt = r / RT, ri = r % RT, kb = k0 >> 5, kk = k0 & 31;
        const int64_t o = ((int64_t)rt * nkb + kb) * (RT * 32) + ((kk >> 3) * (RT >> 3) + (ri >> 3)) * 64 +
                          (ri & 7) * 8;
        uint32_t packed[S][4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
            int d0[S], d1[S];
            digits<S>(t[rr][k0 + j], ex[rr], d0);
            digits<S>(t[rr][k0 + j + 1], ex[rr], d1);
#pragma unroll
            for (int p = 0; p < S; ++p) {
                // w_p = d * 2^(-7p) is exact in bf16 (|d| <= 128)
                const __nv_bfloat162 v = __floats2bfloat162_rn((float)d0[p] * w7[p], (float)d1[p] * w7[p]);
                packed[p][j >> 1] = *reinterpret_cast<const uint32_t*>(&v);
            }
        }
#pragma unroll
        for (int p = 0; p < S; ++p)
            *reinterpret_cast<uint4*>(out + p * slice + o) =
                make_uint4(packed[p][0], packed[p][1], packed[p][2], packed[p][3]);
    }
}

// ---------------------------------------------------------------- tcgen05 GEMM

struct TcProb {
    const __nv_bfloat16* A;  // [S][Mpad][Kpad]
    const __nv_bfloat16* B;  // [S][Npad][Kpad]
    const int32_t* eA;
    const int32_t* eB;
    const double* Cin;
    double* Cout;
    int64_t strideA, strideB, strideEA, strideEB, strideCin, strideC;
    int64_t ldcin, ldc;
    double alpha, beta;
    int32_t M, N, Mpad, Npad, Kpad;
    int32_t batch;
    int32_t lower_only, transCin;
    int32_t tiles_m, tiles_n, tile_begin;
};

struct TcLaunch {
    TcProb p[kMaxTcProbs];
    int32_t np;
    int32_t ks;    // CTAs per output tile (a cluster), each over a K slice
    int32_t* err;  // set to SGB_ERR_TIMEOUT if a bounded wait gave up
    long long spin;  // poll limit of the pipeline's mbarrier waits
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor, no swizzle, K-major.
// bits 0-13 start>>4, 16-29 LBO>>4 (K-direction core-matrix stride),
// 32-45 SBO>>4 (M/N-direction core-matrix stride), 46-47 version = 1,
// 61-63 layout = 0 (no swizzle).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3fff);
    d |= (uint64_t)((lbo >> 4) & 0x3fff) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3fff) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N>>3 at bit 17, M>>4 at bit 24.
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint32_t addr, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t addr, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: returns false if the phase did not complete in `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity, long long limit) {
    for (long long i = 0; i < limit; ++i)
        if (mbar_try(addr, parity)) return true;
    return false;
}


__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accum) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

// 16 consecutive TMEM columns of this warp's 32 lanes; the caller issues
// tmem_wait_ld before using the values (several loads share one wait).
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// The NACC level accumulators of 16 columns (one wait for all of them).
template <int NACC, int BN>
__device__ __forceinline__ void tmem_levels16(uint32_t ta, float (&v)[NACC][16]) {
#pragma unroll
    for (int l = 0; l < NACC; ++l) tmem_ld16_async(ta + l * BN, v[l]);
    tmem_wait_ld();
}

// 16 bytes from the shared memory of a CTA of this cluster (raddr 16-byte aligned).
__device__ __forceinline__ float4 ld_dsmem4(uint32_t raddr) {
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(raddr)
                 : "memory");
    return v;
}

// FP32 -> FP64 by bit operations (exact; zero and subnormal inputs give 0):
// keeps the conversion off the FP64 pipe.
__device__ __forceinline__ double f32_to_f64(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t ex = (u >> 23) & 0xffu;
    if (ex == 0u) return 0.0;
    const uint32_t hi = (u & 0x80000000u) | ((ex + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    const uint32_t lo = (u & 0x7u) << 29;
    return __hiloint2double((int)hi, (int)lo);
}

// r * 2^e on the exponent bits when the result stays normal, else ldexp.
__device__ __forceinline__ double scale_pow2(double r, int e) {
    const long long bits = __double_as_longlong(r);
    const int ex = (int)((bits >> 52) & 0x7ff);
    if (ex == 0) return r;  // zero
    const int nx = ex + e;
    if (nx > 0 && nx < 2047) return __longlong_as_double(bits + ((long long)e << 52));
    return ldexp(r, e);
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t addr, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(addr), "r"(bytes) : "memory");
}

// 1-D bulk copy global -> shared, completing `bytes` on the mbarrier.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(mbar)
        : "memory");
}

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Address of `local_addr` in the shared memory of CTA `rank` of this cluster.
__device__ __forceinline__ uint32_t dsmem_addr(uint32_t local_addr, uint32_t rank) {
    uint32_t raddr;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(raddr) : "r"(local_addr), "r"(rank));
    return raddr;
}

__device__ __forceinline__ float ld_dsmem(uint32_t raddr) {
    float v;
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(raddr) : "memory");
    return v;
}

template <int S, int BN>
struct TcSmem {
    static constexpr int kA = S * TC_BM * TC_BK * 2;   // bytes of A slices per stage
    static constexpr int kB = S * BN * TC_BK * 2;      // bytes of B slices per stage
    static constexpr int kStage = kA + kB;
    static constexpr int kBudget = 225 * 1024;
    static constexpr int kStages = (kBudget / kStage) > 4 ? 4 : (kBudget / kStage);
    static constexpr int kNacc = S < 6 ? S : 6;
    // the epilogue stages the FP64 tile (row stride BN + 1) in the idle
    // stage memory; a K-split CTA keeps its FP32 level accumulators there
    // too and stages only its (at most half of the) rows
    static constexpr int kOut = TC_BM * (BN + 1) * 8;
    static constexpr int kRed = kNacc * TC_BM * BN * 4 + (TC_BM / 2) * (BN + 1) * 8;
    static_assert(kOut <= kStages * kStage, "staging fits the stage memory");
    static constexpr int kData = kStages * kStage > kRed ? kStages * kStage : kRed;
    static constexpr int kExOff = kData + 256;  // staged row / column exponents
    static constexpr int kBytes = kData + 1024 + 1024;
    static_assert(kBytes <= 227 * 1024, "shared memory per CTA");
    static_assert(kStages >= 2, "at least two pipeline stages");
};

// Warp roles (256 threads): warp 4 producer (bulk copies into a kStages
// ring), warp 5 MMA issuer, warps 0-3 wait for the last commit; then all
// eight warps run the epilogue -- each reads the TMEM lanes of its quarter
// (warps w and w + 4 split the columns) -- and share the cross-CTA
// reduction and FP64 writes (measured at n=256, b=512, a=64: pobtaf 87.1 -> 86.3 ms,
// pobtasi 29.8 -> 28.8 ms against six warps; the reduction's ~7 µs are
// spent waiting on its FP64 conversions and stores, not on the distributed
// shared-memory loads, and an integer-only conversion measured slower).
constexpr int TC_THREADS2 = 256;  // warps 6-7 join only the epilogue
static_assert(TC_THREADS2 == 256, "the epilogue's folding splits the columns over two groups of four warps");

template <int S, int BN>
__global__ void __launch_bounds__(TC_THREADS2, 1) k_gemm_tc(const __grid_constant__ TcLaunch L) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    using SM = TcSmem<S, BN>;
    constexpr int NS = SM::kStages;
    uint64_t* full = (uint64_t*)(smem + SM::kData);
    uint64_t* empty = full + NS;
    uint64_t* done = empty + NS;
    uint32_t* tmem_slot = (uint32_t*)(done + 1);
    int* flags = (int*)(tmem_slot + 1);  // [0] error seen, [1] K blocks the producer issued

    const int ks = L.ks;  // CTAs of this tile's cluster, one K slice each
    const uint32_t rank = ks > 1 ? cluster_rank() : 0u;
    const int tile = blockIdx.x / ks;
    int pi = 0;
#pragma unroll 1
    for (int q = 1; q < L.np; ++q)
        if (tile >= L.p[q].tile_begin) pi = q;
    const TcProb& P = L.p[pi];
    int local = tile - P.tile_begin;
    const int per = P.tiles_m * P.tiles_n;
    const int inst = local / per;
    local -= inst * per;
    const int mt = local / P.tiles_n, ntile = local % P.tiles_n;
    const int m0 = mt * TC_BM, n0 = ntile * BN;
    if (P.lower_only && n0 >= m0 + TC_BM) return;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int NACC = S < 6 ? S : 6;
    constexpr int kUsed = NACC * BN;
    constexpr int kCols = kUsed <= 32 ? 32 : kUsed <= 64 ? 64 : kUsed <= 128 ? 128 : kUsed <= 256 ? 256 : 512;
    static_assert(kUsed <= 512, "TMEM columns");

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 32) {
        for (int i = 0; i < NS; ++i) {
            mbar_init(smem_u32(&full[i]), 1);
            mbar_init(smem_u32(&empty[i]), 1);
        }
        mbar_init(smem_u32(done), 1);
        flags[0] = 0;
        flags[1] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    pdl_enter();

    const int nkb_all = P.Kpad / TC_BK;
    const int kb0 = (int)((int64_t)rank * nkb_all / ks), kb1 = (int)((int64_t)(rank + 1) * nkb_all / ks);
    const int nkb = kb1 - kb0;  // this CTA's K slice
    const uint32_t sbase = smem_u32(smem);
    // chunk bases: A chunk (p, mt, kb) and B chunk (q, ntile, kb)
    const unsigned char* Ag = (const unsigned char*)(P.A + (int64_t)inst * P.strideA);
    const unsigned char* Bg = (const unsigned char*)(P.B + (int64_t)inst * P.strideB);
    const int64_t a_slice = (int64_t)P.Mpad * P.Kpad * 2, b_slice = (int64_t)P.Npad * P.Kpad * 2;
    const int64_t a_tile = ((int64_t)mt * nkb_all + kb0) * (TC_BM * TC_BK * 2);
    const int64_t b_tile = ((int64_t)ntile * nkb_all + kb0) * (BN * TC_BK * 2);

    if (warp == 4) {
        // producer
        if (lane == 0) {
            int issued = 0;
            for (int kb = 0; kb < nkb; ++kb) {
                const int st = kb % NS, round = kb / NS;
                if (kb >= NS && !mbar_wait(smem_u32(&empty[st]), (uint32_t)((round - 1) & 1), L.spin)) {
                    atomicExch(&flags[0], 1);
                    break;
                }
                issued = kb + 1;
                const uint32_t fb = smem_u32(&full[st]);
                mbar_expect_tx(fb, (uint32_t)SM::kStage);
                const uint32_t sA = sbase + st * SM::kStage, sB = sA + SM::kA;
#pragma unroll 1
                for (int p = 0; p < S; ++p) {
                    bulk_g2s(sA + p * (TC_BM * TC_BK * 2), Ag + p * a_slice + a_tile + (int64_t)kb * (TC_BM * TC_BK * 2),
                             TC_BM * TC_BK * 2, fb);
                    bulk_g2s(sB + p * (BN * TC_BK * 2), Bg + p * b_slice + b_tile + (int64_t)kb * (BN * TC_BK * 2),
                             BN * TC_BK * 2, fb);
                }
            }
            flags[1] = issued;
        }
    } else if (warp == 5) {
        // MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = make_idesc(TC_BM, BN);
            uint32_t inited = 0;
            for (int kb = 0; kb < nkb; ++kb) {
                const int st = kb % NS, round = kb / NS;
                if (!mbar_wait(smem_u32(&full[st]), (uint32_t)(round & 1), L.spin) || flags[0]) {
                    atomicExch(&flags[0], 1);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t sA = sbase + st * SM::kStage, sB = sA + SM::kA;
#pragma unroll
                for (int ks = 0; ks < TC_BK / 16; ++ks) {
#pragma unroll
                    for (int p = 0; p < S; ++p) {
                        const uint64_t ad = make_desc(sA + p * (TC_BM * TC_BK * 2) + ks * 2 * (TC_BM / 8) * 128,
                                                      (TC_BM / 8) * 128, 128);
#pragma unroll
                        for (int q = 0; q + p < S; ++q) {
                            const int l = (p + q) < NACC ? (p + q) : NACC - 1;
                            const uint64_t bd = make_desc(sB + q * (BN * TC_BK * 2) + ks * 2 * (BN / 8) * 128,
                                                          (BN / 8) * 128, 128);
                            tc_mma(tmem + l * BN, ad, bd, idesc, (inited >> l) & 1u);
                            inited |= 1u << l;
                        }
                    }
                }
                tc_commit(smem_u32(&empty[st]));  // frees the stage when these MMAs finish
            }
            tc_commit(smem_u32(done));  // all issued MMAs
        }
    }

    // epilogue: the level sums of every element become one FP64 value
    // (exact two-sum of the FP32 accumulators, integer widening, one FP64
    // add, power-of-two scale), staged row-major in shared memory, then
    // written out -- alpha, beta and C_in applied -- with consecutive
    // threads on consecutive columns, so global loads and stores coalesce.
    // every warp reads TMEM in the epilogue: each observes the last commit
    // itself, then orders its tcgen05 loads after it
    bool ok = true;
    if (!mbar_wait(smem_u32(done), 0, L.spin)) ok = false;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool all_ok = !__syncthreads_or(!ok || flags[0] != 0);
    if (!all_ok && tid == 0 && L.err != nullptr) atomicExch(L.err, SGB_ERR_TIMEOUT);
    double* C = P.Cout + (int64_t)inst * P.strideC;
    const double* Ci = P.Cin ? P.Cin + (int64_t)inst * P.strideCin : nullptr;
    // the tile's row and column exponents, staged once
    int* eAs = (int*)(smem + SM::kExOff);
    int* eBs = eAs + TC_BM;
    {
        const int32_t* eA = P.eA + (int64_t)inst * P.strideEA;
        const int32_t* eB = P.eB + (int64_t)inst * P.strideEB;
        if (tid < TC_BM) eAs[tid] = (m0 + tid < P.M) ? eA[m0 + tid] : 0;
        else if (tid - TC_BM < BN) eBs[tid - TC_BM] = (n0 + tid - TC_BM < P.N) ? eB[n0 + tid - TC_BM] : 0;
    }
    __syncthreads();
    // FP32 pair hi + lo of a sum: exact two-sum of every term into hi,
    // the rounding errors and small terms collected in lo, then normalised
    auto add2 = [](float& hi, float& lo, float x) {
        const float s2 = hi + x;
        const float bb = s2 - hi;
        lo += (hi - (s2 - bb)) + (x - bb);
        hi = s2;
    };
    auto norm2 = [](float& hi, float& lo) {
        const float h2 = hi + lo;
        lo = lo - (h2 - hi);
        hi = h2;
    };
    // a row of op(A) or column of op(B) holding an Inf or NaN (biased
    // exponent 2047: its digits carry no value) makes the element NaN, as
    // the FP64 product would; a zero row or column otherwise gives 0
    auto finish = [&](float hi, float lo, int eAm, int eBn) -> double {
        if (eAm == 0x7ff || eBn == 0x7ff) return __longlong_as_double(0x7ff8000000000000ll);
        if (eAm == 0 || eBn == 0) return 0.0;
        return scale_pow2(f32_to_f64(hi) + f32_to_f64(lo), eAm + eBn - 2058);
    };
    auto combine = [&](const float (&vv)[NACC], int eAm, int eBn) -> double {
        float hi = vv[0], lo = 0.f;
#pragma unroll
        for (int l = 1; l < NACC; ++l) add2(hi, lo, vv[l]);
        norm2(hi, lo);
        return finish(hi, lo, eAm, eBn);
    };
    const bool neg = P.alpha == -1.0, unit = P.alpha == 1.0 || neg;
    // alpha, beta and C_in applied to one finished element
    auto store = [&](int row, int col, double r) {
        const int m = m0 + row, n = n0 + col;
        if (m >= P.M || n >= P.N || (P.lower_only && n > m)) return;
        if (!unit) r *= P.alpha;
        else if (neg) r = -r;
        if (Ci != nullptr && P.beta != 0.0) {
            const double cv = P.transCin ? Ci[(int64_t)n * P.ldcin + m] : Ci[(int64_t)m * P.ldcin + n];
            r = fma(P.beta, cv, r);
        }
        C[(int64_t)m * P.ldc + n] = r;
    };
    if (ks > 1) {
        // K split over the cluster: each CTA folds its level accumulators of
        // every element into an FP32 pair hi + lo (exact level sums, the
        // pair good to ~2^-48 of the partial -- far below the 2^-(7S+1)
        // slice truncation) and parks the pairs in its (now idle) stage
        // memory as R2[row][col] (row stride BN + 2 pairs, 16-byte stores);
        // after a cluster barrier CTA q sums rows [q*nq, (q+1)*nq) over all
        // CTAs through distributed shared memory, two elements per 16-byte
        // load, every load of a group in flight together, and writes them
        // out, consecutive threads on consecutive column pairs.
        constexpr int LD2 = BN + 2;
        float2* R2 = (float2*)smem;
        if (all_ok) {
            // every warp folds: warp w reads TMEM lanes 32 (w % 4) .. + 31, warps
            // 0-3 the first half of the columns, warps 4-7 the second
            const int q4 = warp & 3, half = warp >> 2;
            const int row = q4 * 32 + lane;
#pragma unroll 1
            for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 16) {
                float v[NACC][16];
                if (nkb > 0) {
                    tmem_levels16<NACC, BN>(tmem + ((uint32_t)(q4 * 32) << 16) + c0, v);
                } else {
#pragma unroll
                    for (int l = 0; l < NACC; ++l)
#pragma unroll
                        for (int i = 0; i < 16; ++i) v[l][i] = 0.f;
                }
#pragma unroll
                for (int i = 0; i < 16; i += 2) {
                    float h0 = v[0][i], l0 = 0.f, h1 = v[0][i + 1], l1 = 0.f;
#pragma unroll
                    for (int l = 1; l < NACC; ++l) {
                        add2(h0, l0, v[l][i]);
                        add2(h1, l1, v[l][i + 1]);
                    }
                    norm2(h0, l0);
                    norm2(h1, l1);
                    *reinterpret_cast<float4*>(&R2[row * LD2 + c0 + i]) = make_float4(h0, l0, h1, l1);
                }
            }
        }
        cluster_sync_all();
        const int nq = (TC_BM + ks - 1) / ks;
        const int r_lo = (int)rank * nq;
        const int nr = (r_lo + nq <= TC_BM ? nq : TC_BM - r_lo);
        uint32_t rb[kTcMaxSplit];
#pragma unroll
        for (int q = 0; q < kTcMaxSplit; ++q) rb[q] = q < ks ? dsmem_addr(smem_u32(R2), (uint32_t)q) : 0u;
        constexpr int G2 = BN / 2;
        if (all_ok) {
#pragma unroll 1
            for (int g = tid; g < nr * G2; g += TC_THREADS2) {
                const int row = r_lo + g / G2, c2 = (g % G2) * 2;
                float4 part[kTcMaxSplit];
#pragma unroll
                for (int q = 0; q < kTcMaxSplit; ++q)
                    part[q] = q < ks ? ld_dsmem4(rb[q] + (uint32_t)((row * LD2 + c2) * 8))
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
                float h0 = part[0].x, l0 = part[0].y, h1 = part[0].z, l1 = part[0].w;
#pragma unroll
                for (int q = 1; q < kTcMaxSplit; ++q) {
                    add2(h0, l0, part[q].x);
                    l0 += part[q].y;
                    add2(h1, l1, part[q].z);
                    l1 += part[q].w;
                }
                norm2(h0, l0);
                norm2(h1, l1);
                store(row, c2, finish(h0, l0, eAs[row], eBs[c2]));
                store(row, c2 + 1, finish(h1, l1, eAs[row], eBs[c2 + 1]));
            }
        }
        cluster_sync_all();  // peers are done reading this CTA's accumulators
    } else {
        // the whole K here: TMEM -> FP64 tile in shared memory -> coalesced writes
        double* Ds = (double*)smem;
        if (all_ok) {
            // as above: all eight warps, two column halves
            const int q4 = warp & 3, half = warp >> 2;
            const int row = q4 * 32 + lane;
            const int eAm = eAs[row];
#pragma unroll 1
            for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 16) {
                float v[NACC][16];
                if (nkb > 0) {
                    tmem_levels16<NACC, BN>(tmem + ((uint32_t)(q4 * 32) << 16) + c0, v);
                } else {
#pragma unroll
                    for (int l = 0; l < NACC; ++l)
#pragma unroll
                        for (int i = 0; i < 16; ++i) v[l][i] = 0.f;
                }
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    float vv[NACC];
#pragma unroll
                    for (int l = 0; l < NACC; ++l) vv[l] = v[l][i];
                    Ds[row * (BN + 1) + c0 + i] = combine(vv, eAm, eBs[c0 + i]);
                }
            }
        }
        __syncthreads();
        if (all_ok) {
#pragma unroll 1
            for (int e = tid; e < TC_BM * BN; e += TC_THREADS2) {
                const int row = e / BN, col = e % BN;
                store(row, col, Ds[row * (BN + 1) + col]);
            }
        }
    }
    if (!all_ok && tid == 0) {
        // drain (bounded by the fixed limit, not the pipeline's): the final
        // commit, then the last round of bulk copies issued into each stage
        // (earlier rounds completed before their stage was refilled)
        mbar_wait(smem_u32(done), 0, kSpinLimit);
        const int issued = flags[1];
        for (int kb = issued > NS ? issued - NS : 0; kb < issued; ++kb)
            mbar_wait(smem_u32(&full[kb % NS]), (uint32_t)((kb / NS) & 1), kSpinLimit);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
    }
}

template <int S, int BN>
cudaError_t set_smem_attr() {
    return cudaFuncSetAttribute(k_gemm_tc<S, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                TcSmem<S, BN>::kBytes);
}

template <int S, int BN>
cudaError_t launch_tc(TcLaunch& L, int total_tiles, cudaStream_t s) {
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3((unsigned)(total_tiles * (L.ks > 1 ? L.ks : 1)));
    cfg.blockDim = dim3(TC_THREADS2);
    cfg.dynamicSmemBytes = TcSmem<S, BN>::kBytes;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    memset(at, 0, sizeof(at));
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    at[1].id = cudaLaunchAttributeClusterDimension;
    at[1].val.clusterDim.x = (unsigned)L.ks;
    at[1].val.clusterDim.y = 1;
    at[1].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = L.ks > 1 ? 2 : 1;
    return cudaLaunchKernelEx(&cfg, k_gemm_tc<S, BN>, L);
}

template <int S>
cudaError_t launch_split(const SplitLaunch& SL, int ctas, cudaStream_t s) {
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3((unsigned)ctas);
    cfg.blockDim = dim3(kSplitThreads);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    memset(at, 0, sizeof(at));
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_split<S>, SL);
}

std::mutex g_attr_mu;
bool g_attr_done[64] = {};

}  // namespace

// ---------------------------------------------------------------- host

cudaError_t tc_prepare() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_attr_mu);
    if (g_attr_done[dev]) return cudaSuccess;
    for (cudaError_t x : {set_smem_attr<3, 64>(), set_smem_attr<4, 64>(), set_smem_attr<5, 64>(),
                          set_smem_attr<6, 64>(), set_smem_attr<7, 64>(), set_smem_attr<3, 32>(),
                          set_smem_attr<4, 32>(), set_smem_attr<5, 32>(), set_smem_attr<6, 32>(),
                          set_smem_attr<7, 32>()})
        if (x != cudaSuccess) return x;
    g_attr_done[dev] = true;
    return cudaSuccess;
}

size_t tc_workspace_bytes(const GemmProb<double>* probs, int np, int S) {
    size_t total = 0;
    for (int i = 0; i < np; ++i) {
        const GemmProb<double>& p = probs[i];
        if (p.M <= 0 || p.N <= 0 || p.batch <= 0) continue;
        int64_t Kpad = 0;
        for (int t = 0; t < p.nterms; ++t) Kpad += ceil_div(p.term[t].K, TC_BK) * TC_BK;
        if (Kpad == 0) Kpad = TC_BK;
        const int64_t Mpad = ceil_div(p.M, TC_BM) * TC_BM;
        const int64_t Npad = ceil_div(p.N, kTcBN) * kTcBN;
        const size_t per = (size_t)S * (Mpad + Npad) * Kpad * 2 + (size_t)(Mpad + Npad) * 4;
        total += (per * p.batch + 255) / 256 * 256 + 256;
    }
    return total;
}

cudaError_t gemm_tc(GemmProb<double>* probs, int np, int S, void* ws, size_t ws_bytes, int32_t* err,
                    cudaStream_t s) {
    if (np > kMaxTcProbs) return cudaErrorInvalidValue;
    if (S != 3 && S != 4 && S != 5 && S != 6 && S != 7) return cudaErrorInvalidValue;
    for (int i = 0; i < np; ++i)
        if (probs[i].nterms > 2) return cudaErrorInvalidValue;  // two sources per split job
    SplitLaunch SL;
    memset(&SL, 0, sizeof(SL));
    SL.S = S;
    TcLaunch TL;
    memset(&TL, 0, sizeof(TL));
    TL.err = err;
    TL.spin = spin_limit();
    char* base = (char*)ws;
    size_t off = 0;
    int64_t split_ctas = 0, gemm_tiles = 0;
    // 128 x 64 tiles.  When they leave most SMs idle, each tile's K range is
    // split over a cluster of ks CTAs (exact FP32 reduction through
    // distributed shared memory); failing that, 128 x 32 tiles.
    // tiles that do work: above-diagonal tiles of a lower-only product exit
    // at once and leave their SMs to the K split of the others
    int64_t tiles64 = 0, minkb = 1 << 30;
    for (int i = 0; i < np; ++i)
        if (probs[i].M > 0 && probs[i].N > 0 && probs[i].batch > 0) {
            const int64_t tm = ceil_div(probs[i].M, TC_BM), tn = ceil_div(probs[i].N, kTcBN);
            int64_t live = tm * tn;
            if (probs[i].lower_only) {
                live = 0;
                for (int64_t m = 0; m < tm; ++m)
                    for (int64_t n = 0; n < tn; ++n) live += (n * kTcBN < (m + 1) * TC_BM) ? 1 : 0;
            }
            tiles64 += live * probs[i].batch;
            int64_t kp = 0;
            for (int t = 0; t < probs[i].nterms; ++t) kp += ceil_div(probs[i].term[t].K, TC_BK);
            minkb = kp < minkb ? kp : minkb;
        }
    int ks = 1;
    // a launch captured beside other streams' work keeps one CTA per tile
    const bool shared_gpu = capture_panel_grid() > 0 && capturing(s) && !capture_tc_split();
    if (tiles64 > 0 && tiles64 < 100 && !shared_gpu) {
        int64_t k = kTcSmCount / tiles64;
        if (k > kTcMaxSplit) k = kTcMaxSplit;
        if (k > minkb) k = minkb;
        ks = k < 1 ? 1 : (int)k;
    }
    const int bn = (ks > 1 || tiles64 >= 148) ? 64 : 32;
    TL.ks = ks;
    for (int i = 0; i < np; ++i) {
        const GemmProb<double>& p = probs[i];
        if (p.M <= 0 || p.N <= 0 || p.batch <= 0) continue;
        int64_t Kpad = 0;
        for (int t = 0; t < p.nterms; ++t) Kpad += ceil_div(p.term[t].K, TC_BK) * TC_BK;
        const int64_t Kalloc = Kpad == 0 ? TC_BK : Kpad;
        if (Kpad > kTcMaxK) return cudaErrorInvalidValue;
        const int64_t Mpad = ceil_div(p.M, TC_BM) * TC_BM;
        const int64_t Npad = ceil_div(p.N, kTcBN) * kTcBN;
        const size_t bytesA = (size_t)S * Mpad * Kalloc * 2, bytesB = (size_t)S * Npad * Kalloc * 2;
        const size_t per = bytesA + bytesB + (size_t)(Mpad + Npad) * 4;
        const size_t per_al = (per + 255) / 256 * 256;
        if (off + per_al * p.batch + 256 > ws_bytes) return cudaErrorInvalidValue;
        __nv_bfloat16* As = (__nv_bfloat16*)(base + off);
        __nv_bfloat16* Bs = (__nv_bfloat16*)(base + off + bytesA);
        int32_t* eA = (int32_t*)(base + off + bytesA + bytesB);
        int32_t* eB = eA + Mpad;
        const int64_t inst_stride_bytes = (int64_t)per_al;
        // split jobs: op(A) rows and op(B) columns, all terms
        SplitJob ja, jb;
        memset(&ja, 0, sizeof(ja));
        memset(&jb, 0, sizeof(jb));
        int32_t koff = 0;
        for (int t = 0; t < p.nterms; ++t) {
            const GemmTerm<double>& tm = p.term[t];
            if (tm.K <= 0) continue;
            SplitSrc& sa = ja.src[ja.nsrc++];
            sa.X = tm.A;
            sa.ld_r = tm.transA ? 1 : tm.lda;
            sa.ld_k = tm.transA ? tm.lda : 1;
            sa.stride = tm.strideA;
            sa.K = tm.K;
            sa.koff = koff;
            SplitSrc& sb = jb.src[jb.nsrc++];
            sb.X = tm.B;
            sb.ld_r = tm.transB ? tm.ldb : 1;
            sb.ld_k = tm.transB ? 1 : tm.ldb;
            sb.stride = tm.strideB;
            sb.K = tm.K;
            sb.koff = koff;
            koff += (int32_t)(ceil_div(tm.K, TC_BK) * TC_BK);
        }
        ja.out = As;
        ja.exps = eA;
        ja.out_stride = inst_stride_bytes / 2;
        ja.exp_stride = inst_stride_bytes / 4;
        ja.R = p.M;
        ja.Rpad = (int32_t)Mpad;
        ja.RT = TC_BM;
        ja.Kpad = (int32_t)Kalloc;
        ja.batch = p.batch;
        ja.strips = (int32_t)(Mpad / kSplitRows);
        jb.out = Bs;
        jb.exps = eB;
        jb.out_stride = ja.out_stride;
        jb.exp_stride = ja.exp_stride;
        jb.R = p.N;
        jb.Rpad = (int32_t)Npad;
        jb.RT = bn;
        jb.Kpad = (int32_t)Kalloc;
        jb.batch = p.batch;
        jb.strips = (int32_t)(Npad / kSplitRows);
        for (SplitJob* j : {&ja, &jb}) {
            if (SL.nj >= kMaxSplitJobs) return cudaErrorInvalidValue;
            j->strip_begin = (int32_t)split_ctas;
            split_ctas += (int64_t)j->strips * j->batch;
            SL.j[SL.nj++] = *j;
        }
        TcProb tp;
        memset(&tp, 0, sizeof(tp));
        tp.A = As;
        tp.B = Bs;
        tp.eA = eA;
        tp.eB = eB;
        tp.Cin = p.Cin;
        tp.Cout = p.Cout;
        tp.strideA = tp.strideB = inst_stride_bytes / 2;
        tp.strideEA = tp.strideEB = inst_stride_bytes / 4;
        tp.strideCin = p.strideCin;
        tp.strideC = p.strideC;
        tp.ldcin = p.ldcin;
        tp.ldc = p.ldc;
        tp.alpha = p.alpha;
        tp.beta = p.beta;
        tp.M = p.M;
        tp.N = p.N;
        tp.Mpad = (int32_t)Mpad;
        tp.Npad = (int32_t)Npad;
        tp.Kpad = (int32_t)Kpad;
        tp.batch = p.batch;
        tp.lower_only = p.lower_only;
        tp.transCin = p.transCin;
        tp.tiles_m = (int32_t)(Mpad / TC_BM);
        tp.tiles_n = (int32_t)(Npad / bn);
        tp.tile_begin = (int32_t)gemm_tiles;
        gemm_tiles += (int64_t)tp.tiles_m * tp.tiles_n * p.batch;
        TL.p[TL.np++] = tp;
        off += per_al * p.batch;
    }
    if (TL.np == 0) return cudaSuccess;
    if (split_ctas > 0) {
        prof_before(s, SGB_KCLASS_SPLIT);
        cudaError_t e;
        switch (S) {
            case 3: e = launch_split<3>(SL, (int)split_ctas, s); break;
            case 4: e = launch_split<4>(SL, (int)split_ctas, s); break;
            case 5: e = launch_split<5>(SL, (int)split_ctas, s); break;
            case 6: e = launch_split<6>(SL, (int)split_ctas, s); break;
            default: e = launch_split<7>(SL, (int)split_ctas, s); break;
        }
        prof_after(SGB_KCLASS_SPLIT, s, 0.0);
        if (e != cudaSuccess) return e;
    }
    double fl = 0.0;
    for (int i = 0; i < np; ++i) fl += useful_flops<double>(probs[i]);
    // bf16 flops the MMA warps issue: every tile that runs (above-diagonal
    // tiles of a lower-only product exit) times its padded K times the
    // S(S+1)/2 slice pairs
    double issued = 0.0;
    for (int i = 0; i < TL.np; ++i) {
        const TcProb& tp = TL.p[i];
        int64_t run = 0;
        for (int mt = 0; mt < tp.tiles_m; ++mt)
            for (int nt = 0; nt < tp.tiles_n; ++nt)
                if (!(tp.lower_only && nt * bn >= mt * TC_BM + TC_BM)) ++run;
        issued += 2.0 * run * tp.batch * (double)TC_BM * bn * tp.Kpad * (S * (S + 1) / 2);
    }
    cudaError_t e = tc_prepare();
    if (e != cudaSuccess) return e;
    prof_before(s, SGB_KCLASS_GEMM_TC);
    if (bn == 64) {
        switch (S) {
            case 3: e = launch_tc<3, 64>(TL, (int)gemm_tiles, s); break;
            case 4: e = launch_tc<4, 64>(TL, (int)gemm_tiles, s); break;
            case 5: e = launch_tc<5, 64>(TL, (int)gemm_tiles, s); break;
            case 6: e = launch_tc<6, 64>(TL, (int)gemm_tiles, s); break;
            default: e = launch_tc<7, 64>(TL, (int)gemm_tiles, s); break;
        }
    } else {
        switch (S) {
            case 3: e = launch_tc<3, 32>(TL, (int)gemm_tiles, s); break;
            case 4: e = launch_tc<4, 32>(TL, (int)gemm_tiles, s); break;
            case 5: e = launch_tc<5, 32>(TL, (int)gemm_tiles, s); break;
            case 6: e = launch_tc<6, 32>(TL, (int)gemm_tiles, s); break;
            default: e = launch_tc<7, 32>(TL, (int)gemm_tiles, s); break;
        }
    }
    prof_after(SGB_KCLASS_GEMM_TC, s, fl, issued);
    return e;
}

}  // namespace sgb
