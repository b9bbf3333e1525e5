/*
 * serinv_gb300 — C ABI of the GB300 (sm_103a) implementation of the
 * sequential block-tridiagonal-with-arrowhead (BTA) hot path:
 *
 *   sgb_pobtaf   block Cholesky            (replaces serinv.algs.pobtaf)
 *   sgb_pobtasi  selected inversion        (replaces serinv.algs.pobtasi)
 *   sgb_pobtas   block triangular solve    (replaces serinv.algs.pobtas)
 *
 * The reference is a Python library without an FFI; each entry point below
 * takes the place of one of its public functions, with the same in-place
 * block-stack layout (C-contiguous, row-major):
 *
 *   diag  (n, b, b)   A_diagonal_blocks        lower triangle meaningful
 *   lower (n-1, b, b) A_lower_diagonal_blocks  lower[i] = A[i+1, i]
 *   arrow (n, a, b)   A_lower_arrow_blocks     arrow[i] = A[tip, i]
 *   tip   (a, a)      A_arrow_tip_block
 *   rhs   (n*b + a, nrhs)
 *
 * All pointers are device pointers (or memory the GPU can address).  Every
 * call is asynchronous on `stream` (a cudaStream_t, 0 = legacy default
 * stream) and allocates nothing: scratch memory comes from the caller as a
 * workspace whose size the matching *_workspace_size query returns.  The
 * return code reports argument and launch errors immediately; a non-SPD
 * pivot is reported on the device through `info` (see below) because it is
 * only known once the kernels have run.
 *
 * Thread safety: calls on different streams with disjoint arrays and
 * workspaces may run concurrently.
 */
#ifndef SERINV_GB300_H
#define SERINV_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes --------------------------------------------------- */
#define SGB_OK               0
#define SGB_ERR_SHAPE        1  /* n < 1, b < 1, a < 0, nrhs < 0, or sizes too large   */
#define SGB_ERR_DTYPE        2  /* dtype not SGB_F32 / SGB_F64                          */
#define SGB_ERR_NOT_SPD      3  /* reported through *info on the device, never returned */
#define SGB_ERR_TIMEOUT      4  /* a bounded device wait gave up                        */
#define SGB_ERR_CUDA         5  /* a CUDA runtime call failed (sgb_last_cuda_error)    */
#define SGB_ERR_WORKSPACE    6  /* workspace missing, too small or misaligned          */
#define SGB_ERR_ARG          7  /* null pointer, bad trans, bad precision              */
#define SGB_ERR_UNSUPPORTED  8  /* valid request this build does not implement         */

/* ---- element types -------------------------------------------------- */
#define SGB_F32 0
#define SGB_F64 1
/* Hermitian positive-definite complex matrices (interleaved re, im pairs,
 * the layout of C99 complex / std::complex / NumPy complex arrays).  They
 * run through the real embedding z = x + iy -> [x -y; y x]: the workspace
 * holds the embedded stacks (twice the matrix's bytes) and the real sweeps
 * run on blocks 2b and arrow 2a.  The imaginary part of the diagonal of the
 * diagonal blocks and of the tip is ignored (taken as 0).  Info rows are
 * complex rows.  SGB_C128 accepts SGB_PREC_MIXED (FP64 embedding). */
#define SGB_C64  2
#define SGB_C128 3

/* ---- precision modes ------------------------------------------------ */
/* Arithmetic in the storage type throughout: the drop-in form. */
#define SGB_PREC_NATIVE 0
/* FP64 storage; the dense block products run on the tensor cores as exact
 * bf16 slice products (fixed-point split of each FP64 operand into S
 * base-128 digits) accumulated exactly in FP32 TMEM and summed in FP64;
 * diagonal-tile pivots stay in FP64.  S goes in bits 8-15 of the precision
 * argument (3..7; 0 selects 6): SGB_PREC_MIXED | (S << 8).  Per-product
 * error ~2^-(7S+1) of the row maxima; measured on pobtaf+pobtasi at
 * n=512, b=512, a=64: S=5 ~4e-9, S=6 ~3e-11, S=7 ~3e-13 relative.
 * FP64 storage only.
 * With S = 7 pobtaf's TRSMs stay FP64 substitutions (the accuracy mode).
 * Bits 16-23 (3..7; 0 = S) set a separate slice count Si for the products
 * with an explicit triangular inverse -- pobtaf's rows-below-the-diagonal
 * times L_ii^{-T}, pobtasi's batched inversions and its products with
 * L_ii^{-1}: SGB_PREC_MIXED | (S << 8) | (Si << 16).  Any explicit Si takes
 * the inverse-based TRSMs, so S = Si = 7 is 7 slices everywhere at nearly
 * the 6-slice speed.
 * The first 4 bytes of the workspace receive a device status word (0, or
 * SGB_ERR_TIMEOUT if a bounded tensor-core wait gave up).                 */
#define SGB_PREC_MIXED  1

typedef struct sgb_bta {
    int32_t dtype;     /* SGB_F32, SGB_F64, SGB_C64 or SGB_C128    */
    int32_t _pad;
    int64_t n;         /* number of diagonal blocks, >= 1          */
    int64_t b;         /* diagonal block size, >= 1                */
    int64_t a;         /* arrowhead width, >= 0                    */
    void* diag;        /* (n, b, b)                                */
    void* lower;       /* (n-1, b, b); may be NULL when n == 1     */
    void* arrow;       /* (n, a, b);  may be NULL when a == 0      */
    void* tip;         /* (a, a);     may be NULL when a == 0      */
} sgb_bta;

/* Library version as 10000*major + 100*minor + patch. */
int sgb_version(void);

/* Static description of a return code. */
const char* sgb_strerror(int code);

/* The cudaError_t of the last SGB_ERR_CUDA returned on this thread. */
int sgb_last_cuda_error(void);

/*
 * Workspace sizes in bytes for one call with these shapes.  The workspace
 * must be device memory aligned to 256 bytes.
 */
int sgb_pobtaf_workspace_size(const sgb_bta* m, int precision, size_t* bytes);
int sgb_pobtasi_workspace_size(const sgb_bta* m, int precision, size_t* bytes);
int sgb_pobtas_workspace_size(const sgb_bta* m, int64_t nrhs, int precision, size_t* bytes);

/*
 * In-place block Cholesky A = L L^T.
 * Replaces serinv.algs.pobtaf (src/serinv/algs/pobtaf.py:11-94, natural
 * ordering _pobtaf :97-183).  On return (stream order) diag holds L_ii with
 * a zero strict upper triangle, lower holds L_{i+1,i}, arrow holds L_{a,i},
 * tip holds L_tip (zero strict upper triangle).
 * factorize_last_block == 0 leaves the last diagonal block and the tip
 * updated but not factorized (pobtaf.py:161).
 * info: device int32 set to 0 at the start of the call and, if a pivot is
 * not positive (or not finite), to the 1-based global row of the first such
 * pivot, like LAPACK potrf.  May be NULL.
 */
int sgb_pobtaf(const sgb_bta* m, int factorize_last_block, int precision,
               void* workspace, size_t workspace_bytes, int32_t* info,
               void* stream);

/*
 * In-place selected inversion from the factor of sgb_pobtaf.
 * Replaces serinv.algs.pobtasi (src/serinv/algs/pobtasi.py:10-89, natural
 * ordering _pobtasi :92-172).  On return diag holds X_ii (full, symmetric),
 * lower holds X_{i+1,i}, arrow holds X_{a,i}, tip holds X_tip: the blocks of
 * A^{-1} on the BTA pattern.  invert_last_block == 0 takes the last diagonal
 * block, the last arrow block and the tip as already inverted
 * (pobtasi.py:114).
 */
int sgb_pobtasi(const sgb_bta* m, int invert_last_block, int precision,
                void* workspace, size_t workspace_bytes, void* stream);

/*
 * In-place block triangular solve with the factor of sgb_pobtaf.
 * Replaces serinv.algs.pobtas (src/serinv/algs/pobtas.py:10-62, natural
 * ordering _pobtas :65-161): trans 'N' computes B <- L^{-1} B, 'T' or 'C'
 * computes B <- L^{-T} B.  rhs is (n*b + a, nrhs) row-major with leading
 * dimension ldb >= nrhs.  partial != 0 skips the last diagonal block and the
 * tip (pobtas.py:99,129).  For a == 0 the call is the arrow-free solve
 * (src/serinv/algs/pobts.py:57-118).
 */
int sgb_pobtas(const sgb_bta* m, void* rhs, int64_t nrhs, int64_t ldb, char trans,
               int partial, int precision, void* workspace, size_t workspace_bytes,
               void* stream);

/*
 * Host-resident stacks (the reference's device_streaming mode, pobtaf.py:
 * 284-524, pobtasi.py:247-496): `host` describes the caller's host arrays
 * (pinned memory for overlap; pageable works, without overlap), `dev` a
 * device copy of the same shape and dtype that the sweep works in (its
 * contents on entry are ignored).  Every block is uploaded on a copy stream
 * in sweep order and downloaded as soon as it is final, overlapped with the
 * factorization or back-sweep; on completion of `stream` the host arrays
 * hold the result, exactly as sgb_pobtaf / sgb_pobtasi leave device arrays.
 * Workspace: sgb_pobtaf_workspace_size / sgb_pobtasi_workspace_size of
 * `dev`.  Real dtypes.
 */
int sgb_pobtaf_host(const sgb_bta* host, const sgb_bta* dev, int factorize_last_block, int precision,
                    void* workspace, size_t workspace_bytes, int32_t* info, void* stream);
int sgb_pobtasi_host(const sgb_bta* host, const sgb_bta* dev, int invert_last_block, int precision,
                     void* workspace, size_t workspace_bytes, void* stream);

/*
 * Host-resident stacks of any size (the reference's device_streaming mode
 * for matrices that do not fit in device memory, pobtaf.py:284-524,
 * pobtasi.py:247-496): `host` describes the caller's host arrays (pinned for
 * overlap).  Only `ring` blocks (D, Lo and Ar of a block per slot) and the
 * tip are on the device at any time: blocks are uploaded on a copy stream
 * ahead of the sweep as slots free up and downloaded once the sweep has read
 * them for the last time, so device memory use does not grow with n.
 * ring <= 0 selects the default (4 for pobtaf, 32 for pobtasi); pobtaf needs
 * ring >= 2, pobtasi an even ring >= 2 (it sweeps chunks of ring/2 blocks).
 * The workspace (size from the matching query, same ring) holds the sweep's
 * scratch, the ring and the tip.  Same results as sgb_pobtaf / sgb_pobtasi
 * on device stacks.  Real dtypes (complex: SGB_ERR_UNSUPPORTED).
 */
int sgb_pobtaf_stream_workspace_size(const sgb_bta* host, int precision, int64_t ring, size_t* bytes);
int sgb_pobtaf_stream(const sgb_bta* host, int factorize_last_block, int precision, int64_t ring,
                      void* workspace, size_t workspace_bytes, int32_t* info, void* stream);
int sgb_pobtasi_stream_workspace_size(const sgb_bta* host, int precision, int64_t ring, size_t* bytes);
int sgb_pobtasi_stream(const sgb_bta* host, int invert_last_block, int precision, int64_t ring,
                       void* workspace, size_t workspace_bytes, void* stream);

/*
 * Permuted (middle-partition) forms: the `buffer=` keyword of the reference
 * functions.  buffer (n, b, b) carries the fill-in between block 0 and the
 * eliminated blocks 1..n-2; blocks 0, n-1 and the tip form the reduced
 * system that the caller factorizes, inverts or solves itself.  n >= 2.
 * SGB_PREC_MIXED (FP64 storage) runs pobtaf's diagonal blocks through the
 * column-block kernel with L_ii^{-T} and every block product on the tensor
 * cores, and pobtasi's products likewise; the solve runs in the storage
 * precision in either mode, as sgb_pobtas does.  The first 4 bytes of the
 * pobtaf / pobtasi workspace receive the device status word.
 *
 * sgb_pobtaf_permuted: pobtaf(..., buffer=) (src/serinv/algs/pobtaf.py:
 *   58-76, _pobtaf_permuted :186-281).  Workspace:
 *   sgb_pobtaf_permuted_workspace_size.  buffer[1] <- lower[0]^H first;
 *   buffer[0] is not touched.
 * sgb_pobtasi_permuted: pobtasi(..., buffer=) (src/serinv/algs/pobtasi.py:
 *   54-71, _pobtasi_permuted :175-244).  On entry blocks 0 and n-1, arrow[0],
 *   arrow[n-1], tip and buffer[n-1] hold the reduced system's inverse.
 *   Workspace: sgb_pobtasi_permuted_workspace_size.
 * sgb_pobtas_permuted: pobtas(..., buffer=) (src/serinv/algs/pobtas.py:
 *   31-46, _pobtas_permuted :164-218).  Workspace:
 *   sgb_pobtas_permuted_workspace_size.
 * For real dtypes the permuted workspace sizes equal the natural ones.
 */
int sgb_pobtaf_permuted(const sgb_bta* m, void* buffer, int precision, void* workspace,
                        size_t workspace_bytes, int32_t* info, void* stream);
int sgb_pobtaf_permuted_workspace_size(const sgb_bta* m, int precision, size_t* bytes);
int sgb_pobtasi_permuted_workspace_size(const sgb_bta* m, int precision, size_t* bytes);
int sgb_pobtas_permuted_workspace_size(const sgb_bta* m, int64_t nrhs, int precision, size_t* bytes);
int sgb_pobtasi_permuted(const sgb_bta* m, void* buffer, int precision, void* workspace,
                         size_t workspace_bytes, void* stream);
int sgb_pobtas_permuted(const sgb_bta* m, void* buffer, void* rhs, int64_t nrhs, int64_t ldb,
                        char trans, int precision, void* workspace, size_t workspace_bytes,
                        void* stream);

/*
 * y <- alpha * A x + beta * y for the symmetric BTA matrix of A's lower
 * stacks (only the lower triangles of diag and tip are read).  x and y are
 * (n*b + a, nrhs) with leading dimensions ldx, ldy >= nrhs and must not
 * overlap (SGB_ERR_ARG).  Real dtypes.  No workspace.
 */
int sgb_bta_symv(const sgb_bta* A, const void* x, int64_t ldx, void* y, int64_t ldy, int64_t nrhs,
                 double alpha, double beta, void* stream);

/*
 * Refined solve: rhs <- A^{-1} rhs with the factor L of A (sgb_pobtaf, any
 * precision) and `iters` steps of iterative refinement against the
 * original A: x = L^{-T} L^{-1} b, then r = b - A x (sgb_bta_symv), x += L^{-T}
 * L^{-1} r.  iters = 0 is the plain solve of sgb_pobtas (N then T).  A and L
 * have the same shape and real dtype.  The reference's pobtas
 * (src/serinv/algs/pobtas.py:10-62) has no refinement; this call serves the
 * mixed-precision factor.
 */
int sgb_pobtas_refine_workspace_size(const sgb_bta* L, int64_t nrhs, size_t* bytes);
int sgb_pobtas_refine(const sgb_bta* A, const sgb_bta* L, void* rhs, int64_t nrhs, int64_t ldb,
                      int iters, void* workspace, size_t workspace_bytes, void* stream);

/*
 * sgb_pobtaf without a workspace argument, for callers that cannot allocate
 * device memory: code running while a stream is being captured, real-time
 * loops that forbid allocator calls, and foreign-language hosts that hold
 * device pointers but no allocator.  This entry point has no counterpart in
 * the reference; it computes exactly what sgb_pobtaf with precision
 * SGB_PREC_NATIVE computes.
 *
 * Its scratch is a static device array of sgb_pobtaf_noalloc_scratch_bytes()
 * bytes (128 KiB) that every GPU loading the library keeps until the process
 * exits.  Requests whose workspace (sgb_pobtaf_workspace_size) exceeds it
 * return SGB_ERR_WORKSPACE.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture.  All calls share the array: calls
 * that overlap on the GPU race and must be serialised by the caller.
 * No cudaMalloc, cudaFree or other allocating routine is called.
 * info (device int32, may be NULL) reports as sgb_pobtaf's does, plus one
 * code of its own: -SGB_ERR_TIMEOUT if a bounded device wait gave up (the
 * status word that sgb_pobtaf leaves in the caller's workspace is private
 * here).  With info NULL a timeout is not reported.
 */
int sgb_pobtaf_noalloc(const sgb_bta* m, int factorize_last_block, int32_t* info, void* stream);
size_t sgb_pobtaf_noalloc_scratch_bytes(void);

/*
 * Row-major C <- alpha op(A) op(B) + beta C in FP64 storage with the same
 * engines the block sweeps use (no counterpart in the reference; it is the
 * dense product every block step of the reference performs with `@`).
 * precision SGB_PREC_NATIVE runs on the FP64 pipe; SGB_PREC_MIXED runs the
 * tensor-core slice products (slice count in bits 8-15 of precision, 3..7,
 * default 6).  transA/transB are 'N' or 'T'.  The first 4 bytes of the
 * workspace receive a device status word (0, or SGB_ERR_TIMEOUT).
 */
int sgb_dgemm_workspace_size(int precision, int64_t M, int64_t N, int64_t K, size_t* bytes);
int sgb_dgemm(int precision, char transA, char transB, int64_t M, int64_t N, int64_t K, double alpha,
              const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
              int64_t ldc, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Backward of logdet(A) + sum_k y_k^T A^{-1} y_k (no counterpart in the
 * reference, which has no differentiation): X holds the selected inverse of
 * A from sgb_pobtasi, x = A^{-1} y is (n*b + a, nrhs) row-major with leading
 * dimension ldx, g points to the upstream gradient (one element of X's
 * dtype, device memory).  In place, X becomes g * dL/d(stored lower stacks):
 * (A^{-1} - x x^T) on the pattern, doubled where a stored entry stands for
 * two entries of the symmetric matrix (strictly-lower entries of diag and
 * tip, every entry of lower and arrow), zero above the diagonal of diag and
 * tip.  Real dtypes; one memory-bound pass, no workspace.
 */
int sgb_bta_logdet_quad_grad(const sgb_bta* X, const void* x, int64_t nrhs, int64_t ldx, const void* g,
                             void* stream);

/* ---- batches of independent matrices ------------------------------------
 * Many BTA matrices of uneven n, b, a and dtype processed by one graph
 * launch (no counterpart in the reference, which handles one matrix per
 * call).  A plan assigns the matrices to `nstreams` concurrent streams
 * (longest first on a cost estimate), captures for every matrix
 *   pobtaf -> pobtas 'N' -> pobtas 'T' -> pobtasi
 * (each present if its bit is in `ops`; the solve uses the factor before
 * the selected inversion overwrites it) into one CUDA graph, and
 * sgb_batch_run replays it on a stream.  rhs[i] is (n*b+a, nrhs[i])
 * row-major; precisions may be NULL (all native).  The workspace (size from
 * sgb_batch_workspace_size with the same arguments) holds one slice per
 * stream and an int32 info word per matrix (sgb_batch_info, device pointer,
 * pobtaf's pivot report).  Plan creation creates and destroys streams and
 * events and builds the graph; sgb_batch_run only launches it.            */
#define SGB_OP_POBTAF  1
#define SGB_OP_POBTASI 2
#define SGB_OP_POBTAS  4

typedef struct sgb_batch_plan sgb_batch_plan;

int sgb_batch_workspace_size(const sgb_bta* mats, void* const* rhs, const int64_t* nrhs, int count,
                             int ops, const int* precisions, int nstreams, size_t* bytes);
int sgb_batch_plan_create(const sgb_bta* mats, void* const* rhs, const int64_t* nrhs, int count, int ops,
                          const int* precisions, int nstreams, void* workspace, size_t workspace_bytes,
                          sgb_batch_plan** plan);
/* As sgb_batch_plan_create, with two schedule parameters for an autotuner:
 * panel_ctas, the CTA count of the captured column-block launches (0
 * selects 24; a count too small for the kernel's roles, < 18, makes those
 * blocks take the launch-based tile sweep), and options: SGB_BATCH_TC_KSPLIT
 * lets the captured tensor-core products split K over thread-block clusters
 * (off by default: the other streams fill the GPU).  The workspace size
 * depends on neither.  Best used with CUDA_DEVICE_MAX_CONNECTIONS >= 32 in
 * the environment (set before the CUDA context exists): the replay's
 * independent branches share that many hardware queues. */
#define SGB_BATCH_TC_KSPLIT 1
int sgb_batch_plan_create_ex(const sgb_bta* mats, void* const* rhs, const int64_t* nrhs, int count, int ops,
                             const int* precisions, int nstreams, int panel_ctas, int options, void* workspace,
                             size_t workspace_bytes, sgb_batch_plan** plan);
int sgb_batch_run(sgb_batch_plan* plan, void* stream);
const int32_t* sgb_batch_info(const sgb_batch_plan* plan);
int sgb_batch_plan_destroy(sgb_batch_plan* plan);

/* ---- diagnostics (no counterpart in the reference) -------------------- */

/* Kernel classes for sgb_profile_read. */
#define SGB_KCLASS_GEMM        0  /* grouped block products (SIMT FP64/FP32)   */
#define SGB_KCLASS_POTRF_TILE  1  /* diagonal-tile Cholesky + tile inverse     */
#define SGB_KCLASS_TRTRI_TILE  2  /* diagonal-tile triangular inverses         */
#define SGB_KCLASS_GEMM_TC     3  /* tensor-core (tcgen05) block products      */
#define SGB_KCLASS_SPLIT       4  /* operand slicing for the tensor-core path  */
#define SGB_KCLASS_PANEL       5  /* persistent column-block Cholesky          */
#define SGB_KCLASS_EMBED       6  /* complex <-> real embedding copies         */
#define SGB_KCLASS_COUNT       7

/* Number of kernels this library has launched since it was loaded. */
long long sgb_launch_count(void);

/* Poll limit of the bounded device waits (the column-block kernel's
 * counters, barriers and staged hand-offs, the tensor-core pipeline's
 * mbarriers); default 2^22 polls, about a second.  Sets the limit for
 * launches made after the call (polls >= 0) and returns the previous one;
 * polls < 0 only queries.  A test hook: a limit of 0 makes every wait that
 * does not find its condition already met give up at once, so the timeout
 * path (status word SGB_ERR_TIMEOUT, every CTA leaving, tensor memory
 * freed) runs without any real hang.  Process-wide; not for production. */
long long sgb_debug_spin_limit(long long polls);

/* Enable (1) or disable (0) per-launch CUDA-event timing; clears records. */
int sgb_profile_enable(int on);

/* Time only the kernel classes in `mask` (bit SGB_KCLASS_*); 0 disables.
 * Events bracket the timed launches only, so the others keep overlapping
 * their neighbours (programmatic dependent launch).  Clears records. */
int sgb_profile_enable_classes(unsigned mask);

/* Totals over the recorded launches of one class: launch count, device
 * milliseconds between the events bracketing each launch, and algorithmic
 * flops (useful multiply-adds x 2).  Synchronises on the recorded events. */
int sgb_profile_read(int kclass, long long* launches, double* ms, double* flops);

/* Arithmetic the hardware issued over the same recorded launches, where it
 * differs from the algorithmic flops: for SGB_KCLASS_GEMM_TC the bf16
 * multiply-adds x 2 of every slice product the MMA warp issues (padding,
 * K splits and all S(S+1)/2 slice pairs included); 0 for other classes. */
int sgb_profile_read_issued(int kclass, double* issued);

#ifdef __cplusplus
}
#endif

#endif /* SERINV_GB300_H */
