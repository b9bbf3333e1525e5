// Internal types shared by the translation units of libserinv_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/serinv_gb300.h"

namespace sgb {

// Diagonal tile width of the blocked Cholesky / triangular inverse.
constexpr int kTile = 32;

// K-range restriction of one product term, for triangular operands.  The
// stored operand must hold exact zeros where the triangle is empty; the
// restriction only skips work.
enum KMode : int8_t {
    KM_FULL = 0,   // k in [0, K)
    KM_GE_N0 = 1,  // op(B) lower triangular: k >= first column of the tile
    KM_LT_N1 = 2,  // op(B) upper triangular: k <  last column of the tile + 1
    KM_GE_M0 = 3,  // op(A) upper triangular: k >= first row of the tile
    KM_LT_M1 = 4,  // op(A) lower triangular: k <  last row of the tile + 1
};

// One product term op(A) * op(B), op(A) is M x K, op(B) is K x N.  A and B
// are row-major with leading dimensions lda / ldb; trans means the stored
// matrix is the transpose of the operand.
template <typename T>
struct GemmTerm {
    const T* A;
    const T* B;
    int64_t lda, ldb;
    int64_t strideA, strideB;  // element stride between batch instances
    int32_t K;
    int8_t transA, transB, kmode, _pad;
};

// Cout = alpha * sum_t op(A_t) op(B_t) + beta * op(Cin), over `batch`
// instances.  Cin may alias Cout when transCin == 0 (each element is read
// and written by the same thread).  A term operand may alias Cout only when
// N <= the tile width (one tile column, rows owned by one CTA).
// Up to three terms per problem (the tensor-core path takes at most two).
constexpr int kMaxTerms = 3;

template <typename T>
struct GemmProb {
    GemmTerm<T> term[kMaxTerms];
    const T* Cin;
    T* Cout;
    int64_t ldcin, ldc;
    int64_t strideCin, strideC;
    T alpha, beta;
    int32_t M, N;
    int32_t nterms;
    int32_t batch;
    int8_t lower_only;  // skip tiles strictly above the diagonal
    int8_t transCin;
    int8_t _pad[2];
    // filled in by the launcher
    int32_t tiles_m, tiles_n, tile_begin;
};

constexpr int kMaxProbs = 6;

template <typename T>
struct GemmLaunch {
    GemmProb<T> p[kMaxProbs];
    int32_t np;
    int32_t total_tiles;
};

// Launch a grouped GEMM (SIMT, arithmetic in T).  Problems with M, N or
// batch of zero are dropped.  Returns cudaSuccess or the launch error.
template <typename T>
cudaError_t gemm_simt(GemmProb<T>* probs, int np, cudaStream_t s);

// Useful flops of one problem (2 x multiply-adds inside the triangles).
template <typename T>
double useful_flops(const GemmProb<T>& p);

// Tile kernels (sgb_potrf.cu).
template <typename T>
cudaError_t potrf_tile(T* tile, int64_t ld, int nb, int zero_cols_right, T* tinv,
                       int32_t* info, int64_t info_row0, cudaStream_t s);

template <typename T>
cudaError_t trtri_tiles_batched(const T* L, int64_t ldl, int64_t strideL, int m, int batch,
                                T* Linv, int64_t ldx, int64_t strideX, cudaStream_t s);

// Blocked in-place Cholesky of the column block [diag; rows_1; ...; rows_k]
// (the diagonal block m x m and up to three row sets with m columns), i.e.
// diag <- chol(diag), rows_j <- rows_j * L^{-T}.  Scratch: kTile*kTile T.
template <typename T>
struct RowSet {
    T* p;
    int64_t rows, ld;
};

template <typename T>
cudaError_t factor_column_block(T* diag, int64_t m, int64_t ldd, RowSet<T> r1, RowSet<T> r2,
                                T* scratch, int32_t* info, int64_t info_row0, cudaStream_t s,
                                RowSet<T> r3 = RowSet<T>{nullptr, 0, 0});

// A grouped-product engine: the SIMT kernel, or a context-bound dispatcher
// that sends products to the tensor cores.
template <typename T>
using GemmFn = cudaError_t (*)(void* ctx, GemmProb<T>* probs, int np, cudaStream_t s);

// The same column-block factorization as one cooperative persistent launch
// (sgb_panel.cu).  `tinv` is 10 * kTile * kTile + 9 * kTile elements of
// scratch, `bar` 16 unsigned words; `status` receives
// SGB_ERR_TIMEOUT if a grid barrier gives up.  With `xinv` (m x m,
// row-major, ld m) the launch also writes L^{-T} there: its upper block
// triangle including the diagonal tiles (zeros below the diagonal inside
// them); the tiles strictly below the diagonal tiles are not written, so
// the caller zeroes them once.  Not for use under stream capture
// (cooperative launch).
// `grid_cap` > 0 limits the grid (a launch captured beside others in a
// graph takes only part of the GPU).
template <typename T>
cudaError_t factor_panel_persistent(T* diag, int64_t m, int64_t ldd, RowSet<T> r1, RowSet<T> r2, T* tinv,
                                    unsigned* bar, int32_t* status, int32_t* info, int64_t info_row0,
                                    cudaStream_t s, T* xinv = nullptr, int grid_cap = 0);

// Grid of the column-block kernel in sweeps captured by this host thread
// (0: captured sweeps use the launch-based tile sweep).  Batch plans set it
// for the duration of their capture; a non-zero value also tells the
// tensor-core products that the captured launches share the GPU with other
// streams (no K split across clusters).
void set_capture_panel_grid(int ctas);
int capture_panel_grid();
// Whether tensor-core products captured beside other streams (a batch
// plan) may split K over clusters; off unless the plan asks for it.
void set_capture_tc_split(bool on);
bool capture_tc_split();

// Full triangular inverse of `batch` lower-triangular m x m blocks:
// Linv_j = L_j^{-1} (zeros above the diagonal).  Scratch: batch*m*m T.
// The row-sweep products go through `fn(fnctx, ...)` when given, else the
// SIMT kernel.
template <typename T>
cudaError_t trtri_batched(const T* L, int64_t ldl, int64_t strideL, int64_t m, int64_t batch,
                          T* Linv, int64_t ldx, int64_t strideX, T* scratch, cudaStream_t s,
                          GemmFn<T> fn = nullptr, void* fnctx = nullptr);

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Tensor-core slice GEMM (sgb_gemm_tc.cu): FP64 storage, exact bf16 slice
// products on tcgen05.  Output tiles 128 x 64 or 128 x 32 (operands are
// padded to kTcBN); the concatenated K of a problem's terms must not exceed
// kTcMaxK (exactness bound of the level accumulators).  `err` (device int32, may be null) receives
// SGB_ERR_TIMEOUT if a bounded wait gives up.
constexpr int kTcBN = 64;
constexpr int kTcMaxK = 576;
size_t tc_workspace_bytes(const GemmProb<double>* probs, int np, int S);
// Sets the tensor-core kernels' shared-memory attribute on the current
// device (once); call before capturing launches into a graph.
cudaError_t tc_prepare();
cudaError_t gemm_tc(GemmProb<double>* probs, int np, int S, void* ws, size_t ws_bytes, int32_t* err,
                    cudaStream_t s);

// y <- alpha A x + beta y for the symmetric BTA matrix of A's lower stacks
// (sgb_refine.cu); x and y (n*b + a rows) must not overlap.
template <typename T>
cudaError_t bta_symv(const sgb_bta* A, const T* x, int64_t ldx, T* y, int64_t ldy, int64_t nrhs, T alpha, T beta,
                     cudaStream_t s);
// x += y over rows x cols.
template <typename T>
cudaError_t axpy2d(T* x, int64_t ldx, const T* y, int64_t ldy, int64_t rows, int64_t cols, cudaStream_t s);

// One matrix of a batch plan (sgb_api.cu): its workspace size and the ops.
size_t plan_item_ws(const sgb_bta* m, int ops, int precision, int64_t nrhs);
int plan_item(const sgb_bta* m, int ops, int precision, void* rhs, int64_t nrhs, void* ws, size_t wsb,
              int32_t* info, cudaStream_t s);

// Records e as this thread's last CUDA error; returns SGB_ERR_CUDA.
int record_cuda_error(cudaError_t e);

// Complex dtypes through the real embedding (sgb_complex.cu).  buffer !=
// nullptr selects the permuted form.
bool cx_dtype(const sgb_bta* m);
int cx_pobtaf_workspace_size(const sgb_bta* m, int precision, size_t* bytes, bool permuted);
int cx_pobtasi_workspace_size(const sgb_bta* m, int precision, size_t* bytes, bool permuted);
int cx_pobtas_workspace_size(const sgb_bta* m, int64_t nrhs, int precision, size_t* bytes, bool permuted);
int cx_pobtaf(const sgb_bta* m, int flb, int precision, void* ws, size_t ws_bytes, int32_t* info, cudaStream_t s,
              void* buffer);
int cx_pobtasi(const sgb_bta* m, int ilb, int precision, void* ws, size_t ws_bytes, cudaStream_t s, void* buffer);
int cx_pobtas(const sgb_bta* m, void* rhs, int64_t nrhs, int64_t ldb, char trans, int partial, int precision,
              void* ws, size_t ws_bytes, cudaStream_t s, void* buffer);

// Poll limit of the bounded device waits (sgb_prof.cu): 2^22 unless a test
// lowered it through sgb_debug_spin_limit.
long long spin_limit();

// Launch accounting (sgb_prof.cu): call prof_before just before and
// prof_after just after every kernel launch.
void prof_before(cudaStream_t s, int kclass = -1);
// True while `s` is being captured into a graph.
bool capturing(cudaStream_t s);
// `issued`: arithmetic the hardware performs for the launch when it differs
// from the algorithmic flops (the tensor-core kernel: bf16 slice products).
void prof_after(int kclass, cudaStream_t s, double flops, double issued = 0.0);

}  // namespace sgb
