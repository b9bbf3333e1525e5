// Complex (Hermitian positive-definite) BTA matrices through the real
// embedding.
//
// Each complex entry z = x + iy becomes the 2 x 2 real block
//     E(z) = [ x  -y ]
//            [ y   x ]
// E is a ring homomorphism (E(zw) = E(z)E(w), E(z^H) = E(z)^T), so for a
// Hermitian positive-definite A with Cholesky factor L (real positive
// diagonal), E(A) = E(L) E(L)^T with E(L) lower triangular with a positive
// diagonal: E(L) is the real Cholesky factor of E(A).  Likewise
// E(A^{-1}) = E(A)^{-1}, so the selected inverse of E(A) on the BTA pattern
// with blocks 2b and arrow 2a is E of the complex selected inverse, and
// E(L)^{-1} (or ^{-T}) applied to the interleaved right-hand side
// [Re x_0; Im x_0; Re x_1; ...] is the interleaved L^{-1} x (or L^{-H} x).
//
// A complex call therefore embeds the stacks into the front of its
// workspace, runs the real sweeps (FP64 or mixed for complex128, FP32 for
// complex64) on the (n, 2b, 2a) real descriptor, and writes the results
// back: Re from entry (2i, 2j) and Im from entry (2i+1, 2j), both in the
// lower triangle of each 2 x 2 block column.  The reference supports
// complex128 throughout (src/serinv/algs/*.py use .conj().T; its tests run
// complex128, tests/conftest.py:18-21); 'T' and 'C' both solve with L^H
// there (pobtas.py:127-159), and here.
//
// Cost: twice the flops of complex arithmetic (8 real per complex
// multiply-add instead of 4) and twice the storage of the stacks, in
// exchange for every real kernel (column-block Cholesky, tensor-core slice
// products) applying unchanged.
#include "sgb_internal.cuh"

namespace sgb {
namespace {

constexpr int kThreads = 256;

template <typename T>
struct Pair;
template <>
struct Pair<double> {
    using V = double2;
};
template <>
struct Pair<float> {
    using V = float2;
};

// dst (count, 2r, 2c) real <- E(src (count, r, c) complex).  herm_diag:
// the stacks are Hermitian diagonal blocks, whose diagonal is real by
// definition; its stored imaginary part is ignored (LAPACK potrf reads the
// real part of the diagonal only).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_embed(const typename Pair<T>::V* __restrict__ src, int64_t count, int64_t r, int64_t c,
            typename Pair<T>::V* __restrict__ dst, int herm_diag) {
    using V = typename Pair<T>::V;
    const int64_t total = count * r * c;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e % c;
        const int64_t ki = e / c;
        const int64_t i = ki % r;
        const int64_t k = ki / r;
        V z = src[e];
        if (herm_diag && i == j) z.y = T(0);
        // rows 2i and 2i+1 of block k, columns 2j, 2j+1 (pairs of T)
        V* row0 = dst + (k * 2 * r + 2 * i) * c;  // in units of V: a real row of 2c T is c V
        row0[j] = V{z.x, -z.y};
        row0[c + j] = V{z.y, z.x};
    }
}

// dst (count, r, c) complex <- entries (2i, 2j) and (2i+1, 2j) of src (count, 2r, 2c).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_compress(const typename Pair<T>::V* __restrict__ src, int64_t count, int64_t r, int64_t c,
               typename Pair<T>::V* __restrict__ dst) {
    using V = typename Pair<T>::V;
    const int64_t total = count * r * c;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e % c;
        const int64_t ki = e / c;
        const int64_t i = ki % r;
        const int64_t k = ki / r;
        const V* row0 = src + (k * 2 * r + 2 * i) * c;
        dst[e] = V{row0[j].x, row0[c + j].x};
    }
}

// Right-hand sides: dst (2N, nrhs) real rows 2r / 2r+1 = Re / Im of row r of
// src (N, nrhs) complex with leading dimension ldb (complex elements).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_embed_rhs(const typename Pair<T>::V* __restrict__ src, int64_t N, int64_t nrhs, int64_t ldb,
                T* __restrict__ dst) {
    const int64_t total = N * nrhs;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / nrhs, j = e - r * nrhs;
        const auto z = src[r * ldb + j];
        dst[(2 * r) * nrhs + j] = z.x;
        dst[(2 * r + 1) * nrhs + j] = z.y;
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_compress_rhs(const T* __restrict__ src, int64_t N, int64_t nrhs, int64_t ldb,
                   typename Pair<T>::V* __restrict__ dst) {
    const int64_t total = N * nrhs;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / nrhs, j = e - r * nrhs;
        dst[r * ldb + j] = typename Pair<T>::V{src[(2 * r) * nrhs + j], src[(2 * r + 1) * nrhs + j]};
    }
}

// info of the real factorization (1-based real row) -> 1-based complex row.
__global__ void k_info_rows(int32_t* info) {
    if (threadIdx.x == 0 && *info > 0) *info = (*info + 1) / 2;
}

unsigned grid_for(int64_t total) {
    int64_t g = (total + kThreads - 1) / kThreads;
    const int64_t cap = 152 * 16;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

bool is_complex(int dtype) { return dtype == SGB_C64 || dtype == SGB_C128; }

// Real descriptor of the embedding (pointers filled in by the layout).
sgb_bta real_desc(const sgb_bta* m) {
    sgb_bta r = *m;
    r.dtype = m->dtype == SGB_C128 ? SGB_F64 : SGB_F32;
    r.b = 2 * m->b;
    r.a = 2 * m->a;
    return r;
}

// Workspace of a complex call: the real call's workspace first (so that its
// status word stays at offset 0), then the embedded stacks.
struct CxLayout {
    size_t real_ws, D, Lo, Ar, T, buf, B, total;
    CxLayout(const sgb_bta& r, size_t real_bytes, bool with_buf, int64_t nrhs) {
        const size_t es = r.dtype == SGB_F64 ? 8 : 4;
        const size_t n = r.n, b = r.b, a = r.a;
        size_t off = 0;
        auto take = [&](size_t bytes) {
            size_t o = off;
            off = align_up(off + bytes);
            return o;
        };
        real_ws = take(real_bytes);
        D = take(es * n * b * b);
        Lo = take(es * (n > 0 ? n - 1 : 0) * b * b);
        Ar = take(es * n * a * b);
        T = take(es * a * a);
        buf = take(with_buf ? es * n * b * b : 0);
        B = take(es * (n * b + a) * (size_t)(nrhs > 0 ? nrhs : 0));
        total = off;
    }
    void point(sgb_bta& r, void* ws) const {
        char* p = (char*)ws;
        r.diag = p + D;
        r.lower = r.n > 1 ? p + Lo : nullptr;
        r.arrow = r.a > 0 ? p + Ar : nullptr;
        r.tip = r.a > 0 ? p + T : nullptr;
    }
};

template <typename T>
cudaError_t embed(const void* src, int64_t count, int64_t rows, int64_t cols, void* dst, int herm, cudaStream_t s) {
    const int64_t total = count * rows * cols;
    if (total <= 0) return cudaSuccess;
    using V = typename Pair<T>::V;
    prof_before(s, SGB_KCLASS_EMBED);
    k_embed<T><<<grid_for(total), kThreads, 0, s>>>((const V*)src, count, rows, cols, (V*)dst, herm);
    prof_after(SGB_KCLASS_EMBED, s, 0.0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t compress(const void* src, int64_t count, int64_t rows, int64_t cols, void* dst, cudaStream_t s) {
    const int64_t total = count * rows * cols;
    if (total <= 0) return cudaSuccess;
    using V = typename Pair<T>::V;
    prof_before(s, SGB_KCLASS_EMBED);
    k_compress<T><<<grid_for(total), kThreads, 0, s>>>((const V*)src, count, rows, cols, (V*)dst);
    prof_after(SGB_KCLASS_EMBED, s, 0.0);
    return cudaGetLastError();
}

int fail(cudaError_t e) { return record_cuda_error(e); }

#define CX_TRY(expr)                               \
    do {                                           \
        cudaError_t _e = (expr);                   \
        if (_e != cudaSuccess) return fail(_e);    \
    } while (0)

// Embeds the four stacks (and buffer / rhs when given) of complex m into the
// workspace; r receives the real descriptor pointing there.
template <typename T>
int embed_all(const sgb_bta* m, sgb_bta& r, const CxLayout& L, void* ws, int herm_diag, const void* buf,
              cudaStream_t s) {
    const int64_t n = m->n, b = m->b, a = m->a;
    L.point(r, ws);
    CX_TRY(embed<T>(m->diag, n, b, b, r.diag, herm_diag, s));
    if (n > 1) CX_TRY(embed<T>(m->lower, n - 1, b, b, r.lower, 0, s));
    if (a > 0) {
        CX_TRY(embed<T>(m->arrow, n, a, b, r.arrow, 0, s));
        CX_TRY(embed<T>(m->tip, 1, a, a, r.tip, herm_diag, s));
    }
    if (buf) CX_TRY(embed<T>(buf, n, b, b, (char*)ws + L.buf, 0, s));
    return SGB_OK;
}

template <typename T>
int compress_all(const sgb_bta* m, const sgb_bta& r, const CxLayout& L, void* ws, void* buf, cudaStream_t s) {
    const int64_t n = m->n, b = m->b, a = m->a;
    CX_TRY(compress<T>(r.diag, n, b, b, m->diag, s));
    if (n > 1) CX_TRY(compress<T>(r.lower, n - 1, b, b, m->lower, s));
    if (a > 0) {
        CX_TRY(compress<T>(r.arrow, n, a, b, m->arrow, s));
        CX_TRY(compress<T>(r.tip, 1, a, a, m->tip, s));
    }
    if (buf) CX_TRY(compress<T>((char*)ws + L.buf, n, b, b, buf, s));
    return SGB_OK;
}

template <typename T>
int rhs_in(const void* rhs, int64_t N, int64_t nrhs, int64_t ldb, void* dst, cudaStream_t s) {
    if (N * nrhs <= 0) return SGB_OK;
    prof_before(s, SGB_KCLASS_EMBED);
    k_embed_rhs<T><<<grid_for(N * nrhs), kThreads, 0, s>>>((const typename Pair<T>::V*)rhs, N, nrhs, ldb, (T*)dst);
    prof_after(SGB_KCLASS_EMBED, s, 0.0);
    CX_TRY(cudaGetLastError());
    return SGB_OK;
}

template <typename T>
int rhs_out(const void* src, int64_t N, int64_t nrhs, int64_t ldb, void* rhs, cudaStream_t s) {
    if (N * nrhs <= 0) return SGB_OK;
    prof_before(s, SGB_KCLASS_EMBED);
    k_compress_rhs<T><<<grid_for(N * nrhs), kThreads, 0, s>>>((const T*)src, N, nrhs, ldb,
                                                              (typename Pair<T>::V*)rhs);
    prof_after(SGB_KCLASS_EMBED, s, 0.0);
    CX_TRY(cudaGetLastError());
    return SGB_OK;
}

int check_ws(void* ws, size_t have, size_t need) {
    if (need == 0) return SGB_OK;
    if (ws == nullptr || have < need) return SGB_ERR_WORKSPACE;
    if (((uintptr_t)ws) % kAlign != 0) return SGB_ERR_WORKSPACE;
    return SGB_OK;
}

}  // namespace

bool cx_dtype(const sgb_bta* m) { return m != nullptr && is_complex(m->dtype); }

// ---- workspace queries -------------------------------------------------

int cx_pobtaf_workspace_size(const sgb_bta* m, int precision, size_t* bytes, bool permuted) {
    sgb_bta r = real_desc(m);
    size_t rb = 0;
    int rc = sgb_pobtaf_workspace_size(&r, precision, &rb);
    if (rc) return rc;
    if (!bytes) return SGB_ERR_ARG;
    *bytes = CxLayout(r, rb, permuted, 0).total;
    return SGB_OK;
}

int cx_pobtasi_workspace_size(const sgb_bta* m, int precision, size_t* bytes, bool permuted) {
    sgb_bta r = real_desc(m);
    size_t rb = 0;
    int rc = permuted ? sgb_pobtasi_permuted_workspace_size(&r, precision, &rb)
                      : sgb_pobtasi_workspace_size(&r, precision, &rb);
    if (rc) return rc;
    if (!bytes) return SGB_ERR_ARG;
    *bytes = CxLayout(r, rb, permuted, 0).total;
    return SGB_OK;
}

int cx_pobtas_workspace_size(const sgb_bta* m, int64_t nrhs, int precision, size_t* bytes, bool permuted) {
    sgb_bta r = real_desc(m);
    size_t rb = 0;
    int rc = sgb_pobtas_workspace_size(&r, nrhs, precision, &rb);
    if (rc) return rc;
    if (!bytes) return SGB_ERR_ARG;
    *bytes = CxLayout(r, rb, permuted, nrhs).total;
    return SGB_OK;
}

// ---- calls ---------------------------------------------------------------

template <typename T>
int cx_pobtaf_t(const sgb_bta* m, int flb, int precision, void* ws, size_t ws_bytes, int32_t* info,
                cudaStream_t s, void* buffer) {
    sgb_bta r = real_desc(m);
    size_t rb = 0;
    int rc = sgb_pobtaf_workspace_size(&r, precision, &rb);
    if (rc) return rc;
    CxLayout L(r, rb, buffer != nullptr, 0);
    if ((rc = check_ws(ws, ws_bytes, L.total))) return rc;
    if ((rc = embed_all<T>(m, r, L, ws, 1, buffer, s))) return rc;
    if (buffer) {
        rc = sgb_pobtaf_permuted(&r, (char*)ws + L.buf, precision, ws, rb, info, s);
    } else {
        rc = sgb_pobtaf(&r, flb, precision, ws, rb, info, s);
    }
    if (rc) return rc;
    if (info) {
        prof_before(s, SGB_KCLASS_EMBED);
        k_info_rows<<<1, 32, 0, s>>>(info);
        prof_after(SGB_KCLASS_EMBED, s, 0.0);
        CX_TRY(cudaGetLastError());
    }
    return compress_all<T>(m, r, L, ws, buffer, s);
}

template <typename T>
int cx_pobtasi_t(const sgb_bta* m, int ilb, int precision, void* ws, size_t ws_bytes, cudaStream_t s, void* buffer) {
    sgb_bta r = real_desc(m);
    size_t rb = 0;
    int rc = buffer ? sgb_pobtasi_permuted_workspace_size(&r, precision, &rb)
                    : sgb_pobtasi_workspace_size(&r, precision, &rb);
    if (rc) return rc;
    CxLayout L(r, rb, buffer != nullptr, 0);
    if ((rc = check_ws(ws, ws_bytes, L.total))) return rc;
    if ((rc = embed_all<T>(m, r, L, ws, 0, buffer, s))) return rc;
    rc = buffer ? sgb_pobtasi_permuted(&r, (char*)ws + L.buf, precision, ws, rb, s)
                : sgb_pobtasi(&r, ilb, precision, ws, rb, s);
    if (rc) return rc;
    return compress_all<T>(m, r, L, ws, buffer, s);
}

template <typename T>
int cx_pobtas_t(const sgb_bta* m, void* rhs, int64_t nrhs, int64_t ldb, char trans, int partial, int precision,
                void* ws, size_t ws_bytes, cudaStream_t s, void* buffer) {
    sgb_bta r = real_desc(m);
    size_t rb = 0;
    int rc = sgb_pobtas_workspace_size(&r, nrhs, precision, &rb);
    if (rc) return rc;
    if (trans != 'N' && trans != 'T' && trans != 'C') return SGB_ERR_ARG;
    if (nrhs < 0 || nrhs > (1 << 20) || ldb < nrhs) return SGB_ERR_SHAPE;
    if ((nrhs > 0 && rhs == nullptr)) return SGB_ERR_ARG;
    CxLayout L(r, rb, buffer != nullptr, nrhs);
    if ((rc = check_ws(ws, ws_bytes, L.total))) return rc;
    if ((rc = embed_all<T>(m, r, L, ws, 0, buffer, s))) return rc;
    const int64_t N = m->n * m->b + m->a;
    void* Br = (char*)ws + L.B;
    if ((rc = rhs_in<T>(rhs, N, nrhs, ldb, Br, s))) return rc;
    const int64_t ldr = nrhs > 0 ? nrhs : 1;
    rc = buffer ? sgb_pobtas_permuted(&r, (char*)ws + L.buf, Br, nrhs, ldr, trans, precision, ws, rb, s)
                : sgb_pobtas(&r, Br, nrhs, ldr, trans, partial, precision, ws, rb, s);
    if (rc) return rc;
    return rhs_out<T>(Br, N, nrhs, ldb, rhs, s);
}

int cx_pobtaf(const sgb_bta* m, int flb, int precision, void* ws, size_t ws_bytes, int32_t* info, cudaStream_t s,
              void* buffer) {
    return m->dtype == SGB_C128 ? cx_pobtaf_t<double>(m, flb, precision, ws, ws_bytes, info, s, buffer)
                                : cx_pobtaf_t<float>(m, flb, precision, ws, ws_bytes, info, s, buffer);
}

int cx_pobtasi(const sgb_bta* m, int ilb, int precision, void* ws, size_t ws_bytes, cudaStream_t s, void* buffer) {
    return m->dtype == SGB_C128 ? cx_pobtasi_t<double>(m, ilb, precision, ws, ws_bytes, s, buffer)
                                : cx_pobtasi_t<float>(m, ilb, precision, ws, ws_bytes, s, buffer);
}

int cx_pobtas(const sgb_bta* m, void* rhs, int64_t nrhs, int64_t ldb, char trans, int partial, int precision,
              void* ws, size_t ws_bytes, cudaStream_t s, void* buffer) {
    return m->dtype == SGB_C128
               ? cx_pobtas_t<double>(m, rhs, nrhs, ldb, trans, partial, precision, ws, ws_bytes, s, buffer)
               : cx_pobtas_t<float>(m, rhs, nrhs, ldb, trans, partial, precision, ws, ws_bytes, s, buffer);
}

}  // namespace sgb
