// Backward of logdet(A) + sum_k y_k^T A^{-1} y_k on the BTA pattern, in place.
//
// dL/dA = A^{-1} - x x^T (x = A^{-1} y), restricted to the pattern and mapped
// to the lower-stack parameterisation: an entry of a stored lower block
// stands for two entries of the symmetric matrix, so strictly-lower entries
// of the diagonal blocks and of the tip, and every entry of the lower and
// arrow blocks, take twice the symmetric-matrix gradient; diagonal entries
// take it once; strictly-upper entries of the diagonal blocks and the tip
// (never read by the factorization) take zero.  The stacks arrive holding
// the selected inverse (pobtasi) and leave holding the gradient times the
// upstream scalar g.  One grid-stride pass: each element reads its inverse
// entry and two rows of x, so the pass is bound by memory traffic.
#include "sgb_internal.cuh"

namespace sgb {
namespace {

template <typename T>
struct GradArgs {
    T* D;
    T* Lo;
    T* Ar;
    T* Tp;
    const T* x;  // (N, k) row-major, leading dimension ldx
    const T* g;  // the upstream gradient (device scalar)
    int64_t n, b, a, k, ldx;
};

template <typename T>
__device__ __forceinline__ T xdot(const GradArgs<T>& p, int64_t r, int64_t c) {
    const T* xr = p.x + r * p.ldx;
    const T* xc = p.x + c * p.ldx;
    T s = T(0);
    for (int64_t q = 0; q < p.k; ++q) s = fma(xr[q], xc[q], s);
    return s;
}

template <typename T>
__global__ void k_pattern_grad(const GradArgs<T> p) {
    const int64_t n = p.n, b = p.b, a = p.a;
    const int64_t bb = b * b, ab = a * b;
    const int64_t nD = n * bb, nLo = (n - 1) * bb, nAr = n * ab, nT = a * a;
    const int64_t total = nD + nLo + nAr + nT;
    const T g = *p.g;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        if (e < nD) {  // D_i (r, c): rows i b + r, i b + c
            const int64_t i = e / bb, rc = e - i * bb, r = rc / b, c = rc - r * b;
            T v = T(0);
            if (c <= r) {
                v = p.D[e] - xdot(p, i * b + r, i * b + c);
                v = (c < r ? T(2) : T(1)) * v * g;
            }
            p.D[e] = v;
        } else if (e < nD + nLo) {  // Lo_i (r, c): rows (i+1) b + r, i b + c
            const int64_t f = e - nD, i = f / bb, rc = f - i * bb, r = rc / b, c = rc - r * b;
            p.Lo[f] = T(2) * (p.Lo[f] - xdot(p, (i + 1) * b + r, i * b + c)) * g;
        } else if (e < nD + nLo + nAr) {  // Ar_i (r, c): rows n b + r, i b + c
            const int64_t f = e - nD - nLo, i = f / ab, rc = f - i * ab, r = rc / b, c = rc - r * b;
            p.Ar[f] = T(2) * (p.Ar[f] - xdot(p, n * b + r, i * b + c)) * g;
        } else {  // T (r, c): rows n b + r, n b + c
            const int64_t f = e - nD - nLo - nAr, r = f / a, c = f - r * a;
            T v = T(0);
            if (c <= r) {
                v = p.Tp[f] - xdot(p, n * b + r, n * b + c);
                v = (c < r ? T(2) : T(1)) * v * g;
            }
            p.Tp[f] = v;
        }
    }
}

template <typename T>
cudaError_t pattern_grad(const sgb_bta* X, const T* x, int64_t k, int64_t ldx, const T* g, cudaStream_t s) {
    GradArgs<T> p;
    p.D = (T*)X->diag;
    p.Lo = (T*)X->lower;
    p.Ar = (T*)X->arrow;
    p.Tp = (T*)X->tip;
    p.x = x;
    p.g = g;
    p.n = X->n;
    p.b = X->b;
    p.a = X->a;
    p.k = k;
    p.ldx = ldx;
    const int64_t total = X->n * X->b * X->b + (X->n - 1) * X->b * X->b + X->n * X->a * X->b + X->a * X->a;
    int64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    prof_before(s);
    k_pattern_grad<T><<<(unsigned)blocks, 256, 0, s>>>(p);
    const cudaError_t e = cudaGetLastError();
    prof_after(-1, s, 0.0);
    return e;
}

}  // namespace
}  // namespace sgb

extern "C" int sgb_bta_logdet_quad_grad(const sgb_bta* X, const void* x, int64_t nrhs, int64_t ldx, const void* g,
                                        void* stream) {
    if (X == nullptr || x == nullptr || g == nullptr) return SGB_ERR_ARG;
    if (X->dtype != SGB_F32 && X->dtype != SGB_F64) return SGB_ERR_DTYPE;
    if (X->n < 1 || X->b < 1 || X->a < 0) return SGB_ERR_SHAPE;
    if (nrhs < 1 || ldx < nrhs) return SGB_ERR_SHAPE;
    if (X->diag == nullptr || (X->n > 1 && X->lower == nullptr) ||
        (X->a > 0 && (X->arrow == nullptr || X->tip == nullptr)))
        return SGB_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const cudaError_t e =
        X->dtype == SGB_F64
            ? sgb::pattern_grad<double>(X, (const double*)x, nrhs, ldx, (const double*)g, s)
            : sgb::pattern_grad<float>(X, (const float*)x, nrhs, ldx, (const float*)g, s);
    return e == cudaSuccess ? SGB_OK : sgb::record_cuda_error(e);
}
