// C ABI entry points: argument checks, workspace layout, and the host-side
// block sweeps of pobtaf / pobtasi / pobtas that enqueue the kernels.
#include <string.h>

#include <vector>

#include "sgb_internal.cuh"

namespace sgb {
namespace {

thread_local int g_last_cuda_error = 0;

int cuda_fail(cudaError_t e) {
    g_last_cuda_error = (int)e;
    return SGB_ERR_CUDA;
}

}  // namespace

int record_cuda_error(cudaError_t e) { return cuda_fail(e); }

namespace {

#define SGB_TRY(expr)                                     \
    do {                                                  \
        cudaError_t _e = (expr);                          \
        if (_e != cudaSuccess) return cuda_fail(_e);      \
    } while (0)

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Largest sizes the 32-bit tile indexing handles comfortably.
constexpr int64_t kMaxBlock = 1 << 16;

int check_bta(const sgb_bta* m) {
    if (m == nullptr) return SGB_ERR_ARG;
    if (m->dtype != SGB_F32 && m->dtype != SGB_F64) return SGB_ERR_DTYPE;
    if (m->n < 1 || m->b < 1 || m->a < 0) return SGB_ERR_SHAPE;
    if (m->b > kMaxBlock || m->a > kMaxBlock || m->n > (int64_t)1 << 30) return SGB_ERR_SHAPE;
    if (m->diag == nullptr) return SGB_ERR_ARG;
    if (m->n > 1 && m->lower == nullptr) return SGB_ERR_ARG;
    if (m->a > 0 && (m->arrow == nullptr || m->tip == nullptr)) return SGB_ERR_ARG;
    return SGB_OK;
}

// precision: SGB_PREC_NATIVE, or SGB_PREC_MIXED with the slice count in
// bits 8-15 (0 = default kDefaultSlices).  Returns the slice count (0 for
// native) or a negative error code.
constexpr int kDefaultSlices = 6;

int parse_precision(int precision, int dtype) {
    const int mode = precision & 0xff;
    if (mode == SGB_PREC_NATIVE && (precision >> 8) == 0) return 0;
    if (mode != SGB_PREC_MIXED) return -SGB_ERR_ARG;
    int S = (precision >> 8) & 0xff;
    if (S == 0) S = kDefaultSlices;
    if (S < 3 || S > 7) return -SGB_ERR_ARG;
    const int Si = (precision >> 16) & 0xff;
    if ((Si != 0 && (Si < 3 || Si > 7)) || (precision >> 24) != 0) return -SGB_ERR_ARG;
    if (dtype != SGB_F64) return -SGB_ERR_UNSUPPORTED;
    return S;
}

// Slice count of the products with an explicit triangular inverse (the
// rows below a diagonal block times L_ii^{-T} in pobtaf; the batched
// inversions and the G, H, P products of pobtasi): bits 16-23 of the
// precision argument; 0 (returned as 0) = the same as S, except that S = 7
// then keeps pobtaf's TRSMs as FP64 substitutions.  An explicit count always
// takes the inverse-based products, so S = Si = 7 is the fast form with
// every product at 7 slices.
int parse_inv_slices(int precision, int S) {
    if (S <= 0) return 0;
    return (precision >> 16) & 0xff;
}

// Everything a block sweep needs besides the matrix: precision and the
// tensor-core scratch carved from the caller's workspace.
struct Ctx {
    int slices = 0;          // 0: native arithmetic; 3..7: tensor-core slice products
    void* tc = nullptr;      // slice buffers
    size_t tc_bytes = 0;
    int32_t* status = nullptr;  // device status word (SGB_ERR_TIMEOUT on a stuck wait)
};


// Upper bound of the tensor-core scratch of one grouped launch with up to
// `nprob` problems whose sizes are at most mx x mx and K at most kmax.
size_t tc_bound(int S, int64_t mx, int64_t kmax, int nprob) {
    const int64_t Mpad = ceil_div(mx, 128) * 128, Npad = ceil_div(mx, kTcBN) * kTcBN;
    const int64_t Kpad = ceil_div(kmax, 32) * 32 + 32;
    const size_t per = (size_t)S * (Mpad + Npad) * Kpad * 2 + (size_t)(Mpad + Npad) * 4;
    return (size_t)nprob * ((per + 255) / 256 * 256 + 256);
}

template <typename T>
cudaError_t run_gemm(const Ctx& c, GemmProb<T>* pr, int np, cudaStream_t s) {
    return gemm_simt<T>(pr, np, s);
}

// FP64: in mixed mode every product with K <= kTcMaxK goes to the tensor
// cores; copies (no product term) and longer K stay on the FP64 pipe.
template <>
cudaError_t run_gemm<double>(const Ctx& c, GemmProb<double>* pr, int np, cudaStream_t s) {
    if (c.slices == 0) return gemm_simt<double>(pr, np, s);
    GemmProb<double> tc[kMaxProbs], simt[kMaxProbs];
    int ntc = 0, nsimt = 0;
    for (int i = 0; i < np; ++i) {
        int64_t kpad = 0;
        for (int t = 0; t < pr[i].nterms; ++t) kpad += ceil_div(pr[i].term[t].K, 32) * 32;
        if (pr[i].nterms > 0 && kpad > 0 && kpad <= kTcMaxK && ntc < 4) tc[ntc++] = pr[i];
        else simt[nsimt++] = pr[i];
    }
    if (ntc) {
        cudaError_t e = gemm_tc(tc, ntc, c.slices, c.tc, c.tc_bytes, c.status, s);
        if (e != cudaSuccess) return e;
    }
    if (nsimt) return gemm_simt<double>(simt, nsimt, s);
    return cudaSuccess;
}

template <typename T>
cudaError_t ctx_gemm(void* c, GemmProb<T>* pr, int np, cudaStream_t s) {
    return run_gemm<T>(*(const Ctx*)c, pr, np, s);
}

// Independent problems of up to three terms each.  Natively one SIMT launch.
// With slices, each problem's terms are cut into groups that fit the
// tensor-core bound (concatenated K <= kTcMaxK, at most two terms); group g
// of every problem goes in round g -- the first with the problem's own beta
// and C_in, the later ones accumulating into C_out -- at most four problems
// per tensor-core launch.
template <typename T>
cudaError_t run_gemm_groups(const Ctx& c, const GemmProb<T>* pr, int np, cudaStream_t s) {
    if (c.slices == 0) {
        GemmProb<T> tmp[kMaxProbs];
        for (int i = 0; i < np; ++i) tmp[i] = pr[i];
        return gemm_simt<T>(tmp, np, s);
    }
    GemmProb<T> rounds[kMaxTerms][kMaxProbs];
    int nr[kMaxTerms] = {0, 0, 0};
    for (int i = 0; i < np; ++i) {
        const GemmProb<T>& p = pr[i];
        int g = 0, t = 0;
        while (t < p.nterms || (t == 0 && p.nterms == 0)) {
            GemmProb<T> q = p;
            q.nterms = 0;
            int64_t k = 0;
            while (t < p.nterms && q.nterms < 2) {
                const int64_t kp = ceil_div(p.term[t].K, 32) * 32;
                if (q.nterms > 0 && k + kp > kTcMaxK) break;
                q.term[q.nterms++] = p.term[t++];
                k += kp;
            }
            if (g > 0) {  // accumulate onto the previous rounds' result
                q.beta = T(1);
                q.Cin = q.Cout;
                q.ldcin = q.ldc;
                q.strideCin = q.strideC;
                q.transCin = 0;
            }
            rounds[g][nr[g]++] = q;
            ++g;
            if (p.nterms == 0) break;
        }
    }
    for (int g = 0; g < kMaxTerms; ++g)
        for (int i0 = 0; i0 < nr[g]; i0 += 4) {
            const int cnt = nr[g] - i0 < 4 ? nr[g] - i0 : 4;
            cudaError_t e = run_gemm<T>(c, rounds[g] + i0, cnt, s);
            if (e != cudaSuccess) return e;
        }
    return cudaSuccess;
}

// Tensor-core scratch of the largest grouped product of a batched
// recursive-doubling inversion of `batch` m x m blocks: at level h, up to
// four pair problems of h x h (K = h) per launch.
size_t trtri_tc_bytes(int S, int64_t m, int64_t batch) {
    size_t best = 0;
    for (int64_t h = kTile; h < m; h *= 2) {
        const int64_t pairs = (m / h + 1) / 2;
        const int64_t group = pairs < 4 ? pairs : 4;
        const int64_t Mpad = ceil_div(h, 128) * 128, Npad = ceil_div(h, kTcBN) * kTcBN, Kpad = ceil_div(h, 32) * 32;
        const size_t per = (size_t)S * (Mpad + Npad) * Kpad * 2 + (size_t)(Mpad + Npad) * 4;
        const size_t bytes = (size_t)group * ((size_t)batch * ((per + 255) / 256 * 256) + 256);
        best = bytes > best ? bytes : best;
    }
    return best + 512;
}

// Blocks per chunk of a batched inversion (bounds the scratch).
constexpr int64_t kTrtriChunk = 64;

int64_t trtri_chunk(int64_t batch) { return batch < kTrtriChunk ? batch : kTrtriChunk; }

// Scratch elements of trtri_run for `batch` m x m blocks.
size_t trtri_scratch_elems(int64_t m, int64_t batch) { return (size_t)trtri_chunk(batch) * m * m; }

// Batched L^{-1} in chunks of kTrtriChunk blocks: SIMT products natively,
// tensor-core products in mixed mode.
template <typename T>
cudaError_t trtri_run(const Ctx& cx, const T* L, int64_t m, int64_t batch, T* Linv, T* scratch, cudaStream_t s) {
    const int64_t mm = m * m;
    for (int64_t j0 = 0; j0 < batch; j0 += kTrtriChunk) {
        const int64_t nb = (batch - j0) < kTrtriChunk ? (batch - j0) : kTrtriChunk;
        cudaError_t e = cx.slices == 0
                            ? trtri_batched<T>(L + j0 * mm, m, mm, m, nb, Linv + j0 * mm, m, mm, scratch, s)
                            : trtri_batched<T>(L + j0 * mm, m, mm, m, nb, Linv + j0 * mm, m, mm, scratch, s,
                                               ctx_gemm<T>, (void*)&cx);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// ---- workspace layouts ------------------------------------------------

struct Carve {
    size_t off = 0;
    size_t take(size_t bytes) {
        size_t o = off;
        off = align_up(off + bytes);
        return o;
    }
};

template <typename T>
struct PobtafWs {
    size_t status, bar, tinv, tc, tc_bytes, xinv, total;
    PobtafWs(const sgb_bta* m, int S = 0, int Si = 0) {
        Carve c;
        status = c.take(256);
        bar = c.take(256);
        tinv = c.take(sizeof(T) * (10 * kTile * kTile + 9 * kTile));  // column-block kernel scratch
        const int64_t mx = m->b > m->a ? m->b : m->a;
        const int Sm = Si > S ? Si : S;
        tc_bytes = S ? tc_bound(Sm, mx, m->b, 4) : 0;  // up to four problems per product launch
        tc = c.take(tc_bytes);
        // mixed precision only: L_ii^{-T} of the current diagonal block
        xinv = c.take(S ? sizeof(T) * m->b * m->b : 0);
        total = c.off;
    }
};

// pobtasi works through the blocks in chunks: L_jj^{-1}, G_j = Lo_j L_jj^{-1},
// H_j = Ar_j L_jj^{-1} and P_j = L_jj^{-T} L_jj^{-1} of a chunk are formed
// by batched products first, then the chunk's back-sweep steps run.
constexpr int64_t kSiChunk = 64;
// Blocks per grouped tensor-core launch of those batched products (bounds
// the slice scratch).
constexpr int64_t kSiTcBatch = 16;

// Slice scratch gemm_tc takes for one problem (sizes as gemm_tc pads them).
size_t tc_prob_bytes(int S, int64_t M, int64_t N, int64_t Kpad, int64_t batch) {
    const int64_t Mpad = ceil_div(M, 128) * 128, Npad = ceil_div(N, kTcBN) * kTcBN;
    const int64_t Kal = Kpad <= 0 ? 32 : ceil_div(Kpad, 32) * 32;
    const size_t per = (size_t)S * (Mpad + Npad) * Kal * 2 + (size_t)(Mpad + Npad) * 4;
    return (per + 255) / 256 * 256 * (size_t)batch + 256;
}

template <typename T>
struct PobtasiWs {
    size_t status, linv, linv_tip, trtri, gh, tc, tc_bytes, total;
    int64_t chunk;
    // chunk_cap: blocks per chunk at most (a streaming ring holds two chunks)
    PobtasiWs(const sgb_bta* m, int S = 0, int Si = 0, int64_t chunk_cap = kSiChunk) {
        const int64_t n = m->n, b = m->b, a = m->a;
        const int64_t cap = chunk_cap < 1 ? 1 : (chunk_cap < kSiChunk ? chunk_cap : kSiChunk);
        chunk = n < cap ? (n > 0 ? n : 1) : cap;
        Carve c;
        status = c.take(256);
        tc_bytes = 0;
        if (Si > S) S = Si;  // scratch for the larger of the two slice counts
        if (S) {
            const int64_t kba = ceil_div(b, 32) * 32 + ceil_div(a, 32) * 32;
            const int64_t tb = chunk < kSiTcBatch ? chunk : kSiTcBatch;
            size_t need[5];
            need[0] = tc_prob_bytes(S, b, b, kba, 1) + tc_prob_bytes(S, a, b, kba, 1);  // back-sweep step
            need[1] = 2 * tc_prob_bytes(S, b, b, b, tb) + tc_prob_bytes(S, a, b, b, tb);  // G, P, H
            need[2] = trtri_tc_bytes(S, b, chunk);
            need[3] = trtri_tc_bytes(S, a, 1);
            need[4] = tc_prob_bytes(S, a, a, a, 1);  // tip
            for (size_t v : need) tc_bytes = v > tc_bytes ? v : tc_bytes;
        }
        tc = c.take(tc_bytes);
        linv = c.take(sizeof(T) * (size_t)(chunk * b * b));
        linv_tip = c.take(sizeof(T) * (size_t)(a * a));
        const size_t t1 = trtri_scratch_elems(b, chunk), t2 = trtri_scratch_elems(a, 1);
        trtri = c.take(sizeof(T) * (t1 > t2 ? t1 : t2));
        gh = c.take(sizeof(T) * (size_t)(chunk * (b + a) * b));
        total = c.off;
    }
};

template <typename T>
struct PobtasWs {
    size_t linv, linv_tip, trtri, y, total;
    PobtasWs(const sgb_bta* m, int64_t nrhs) {
        const size_t n = m->n, b = m->b, a = m->a;
        const size_t mx = b > a ? b : a;
        Carve c;
        linv = c.take(sizeof(T) * n * b * b);
        linv_tip = c.take(sizeof(T) * a * a);
        trtri = c.take(sizeof(T) * trtri_scratch_elems((int64_t)mx, (int64_t)n));
        y = c.take(sizeof(T) * mx * (size_t)nrhs);
        total = c.off;
    }
};

int check_ws(void* ws, size_t have, size_t need) {
    if (need == 0) return SGB_OK;
    if (ws == nullptr || have < need) return SGB_ERR_WORKSPACE;
    if (((uintptr_t)ws) % kAlign != 0) return SGB_ERR_WORKSPACE;
    return SGB_OK;
}

template <typename T>
GemmProb<T> prob() {
    GemmProb<T> p;
    memset(&p, 0, sizeof(p));
    p.batch = 1;
    p.alpha = T(1);
    return p;
}

template <typename T>
void set_term(GemmProb<T>& p, int t, const T* A, int64_t lda, int transA, const T* B, int64_t ldb, int transB,
              int64_t K, int kmode = KM_FULL) {
    p.term[t].A = A;
    p.term[t].lda = lda;
    p.term[t].transA = (int8_t)transA;
    p.term[t].B = B;
    p.term[t].ldb = ldb;
    p.term[t].transB = (int8_t)transB;
    p.term[t].K = (int32_t)K;
    p.term[t].kmode = (int8_t)kmode;
    if (t + 1 > p.nterms) p.nterms = t + 1;
}

// Copy problem: Cout = Cin (M x N).
template <typename T>
GemmProb<T> copy_prob(T* dst, int64_t ldd, const T* src, int64_t lds, int64_t M, int64_t N) {
    GemmProb<T> p = prob<T>();
    p.M = (int32_t)M;
    p.N = (int32_t)N;
    p.alpha = T(0);
    p.beta = T(1);
    p.Cin = src;
    p.ldcin = lds;
    p.Cout = dst;
    p.ldc = ldd;
    return p;
}

// ---- block addresses -------------------------------------------------------
// Block i's diagonal, lower and arrow blocks: in the stacks themselves, or in
// a device ring of R slots (host-resident stacks streamed through HBM), slot
// (i - off) mod R.  Batched operations over blocks lo..hi-1 need them in
// consecutive slots (contiguous()).
template <typename T>
struct Blocks {
    T* D = nullptr;
    T* Lo = nullptr;
    T* Ar = nullptr;
    int64_t bb = 0, ab = 0;
    int64_t R = 0, off = 0;
    int64_t slot(int64_t i) const {
        if (R == 0) return i;
        const int64_t r = (i - off) % R;
        return r < 0 ? r + R : r;
    }
    T* d(int64_t i) const { return D + slot(i) * bb; }
    T* lo(int64_t i) const { return Lo + slot(i) * bb; }
    T* ar(int64_t i) const { return Ar + slot(i) * ab; }
    bool contiguous(int64_t lo_, int64_t hi) const {
        return R == 0 || hi <= lo_ || (hi - lo_ <= R && slot(hi - 1) - slot(lo_) == hi - 1 - lo_);
    }
};

// How a sweep's blocks reach the device when the caller's stacks are in host
// memory.  The sweep calls need(i) before it reads block i, give(i) once
// block i holds its final values, release(i) once it will not read block i
// again, give_tip() once the tip is final, and finish() at the end.
struct Link {
    virtual ~Link() = default;
    virtual cudaError_t start(cudaStream_t s) = 0;
    virtual cudaError_t need(int64_t i, cudaStream_t s) = 0;
    virtual cudaError_t give(int64_t i, cudaStream_t s) = 0;
    virtual cudaError_t release(int64_t i, cudaStream_t s) = 0;
    virtual cudaError_t give_tip() = 0;
    virtual cudaError_t finish(cudaStream_t s) = 0;
};

// ---- host-resident stacks --------------------------------------------------
// The stacks live in host memory (pinned for overlap) and are staged in a
// device copy of the same shape.  Uploads of every block are enqueued up
// front on a copy stream in the order the sweep consumes them, with an event
// per group of kLinkGroup blocks; the sweep waits for a group's event only
// when it reaches the group.  Finished blocks go back on a second copy
// stream a group at a time, ordered after the launches that finalised them.
// The transfers overlap the factorization / back-sweep, so a host-array call
// costs little more than the device-resident one.
constexpr int64_t kLinkGroup = 8;

struct HostLink : Link {
    const sgb_bta* h = nullptr;  // host stacks
    const sgb_bta* d = nullptr;  // device stacks (same shape)
    bool ascending = true;       // sweep order: pobtaf ascending, pobtasi descending
    size_t es = 8;
    cudaStream_t up = nullptr, down = nullptr;
    std::vector<cudaEvent_t> up_ev, events;
    int64_t waited = -1;
    std::vector<int64_t> pending;
    bool tip_pending = false;

    cudaError_t event(cudaEvent_t* e) {
        cudaError_t r = cudaEventCreateWithFlags(e, cudaEventDisableTiming);
        if (r == cudaSuccess) events.push_back(*e);
        return r;
    }
    cudaError_t copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st) {
        return bytes ? cudaMemcpyAsync(dst, src, bytes, kind, st) : cudaSuccess;
    }
    cudaError_t block(int64_t i, bool to_dev, cudaStream_t st) {
        const int64_t n = h->n, b = h->b, a = h->a;
        const cudaMemcpyKind k = to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
        auto mv = [&](void* hb, void* db, int64_t off, int64_t cnt) {
            char* hp = (char*)hb + es * off;
            char* dp = (char*)db + es * off;
            return to_dev ? copy(dp, hp, es * cnt, k, st) : copy(hp, dp, es * cnt, k, st);
        };
        cudaError_t r = mv(h->diag, d->diag, i * b * b, b * b);
        if (r == cudaSuccess && i < n - 1) r = mv(h->lower, d->lower, i * b * b, b * b);
        if (r == cudaSuccess && a) r = mv(h->arrow, d->arrow, i * a * b, a * b);
        return r;
    }
    cudaError_t tip(bool to_dev, cudaStream_t st) {
        const int64_t a = h->a;
        if (!a) return cudaSuccess;
        return to_dev ? copy(d->tip, h->tip, es * a * a, cudaMemcpyHostToDevice, st)
                      : copy(h->tip, d->tip, es * a * a, cudaMemcpyDeviceToHost, st);
    }
    int64_t pos(int64_t i) const { return ascending ? i : h->n - 1 - i; }

    // Enqueue every upload (the tip first) after the work already on s.
    cudaError_t start(cudaStream_t s) override {
        cudaError_t r = cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking);
        if (r == cudaSuccess) r = cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking);
        cudaEvent_t e0;
        if (r == cudaSuccess) r = event(&e0);
        if (r == cudaSuccess) r = cudaEventRecord(e0, s);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(up, e0, 0);
        if (r == cudaSuccess) r = tip(true, up);
        const int64_t n = h->n;
        for (int64_t p = 0; p < n && r == cudaSuccess; ++p) {
            r = block(ascending ? p : n - 1 - p, true, up);
            if (r == cudaSuccess && ((p + 1) % kLinkGroup == 0 || p == n - 1)) {
                cudaEvent_t e;
                r = event(&e);
                if (r == cudaSuccess) r = cudaEventRecord(e, up);
                if (r == cudaSuccess) up_ev.push_back(e);
            }
        }
        return r;
    }
    // Block i (and every block before it in sweep order, and the tip) resident.
    cudaError_t need(int64_t i, cudaStream_t s) override {
        const int64_t g = pos(i) / kLinkGroup;
        if (g <= waited) return cudaSuccess;
        waited = g;
        return cudaStreamWaitEvent(s, up_ev[(size_t)g], 0);
    }
    cudaError_t flush(cudaStream_t s) {
        if (pending.empty() && !tip_pending) return cudaSuccess;
        cudaEvent_t e;
        cudaError_t r = event(&e);
        if (r == cudaSuccess) r = cudaEventRecord(e, s);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(down, e, 0);
        for (int64_t i : pending)
            if (r == cudaSuccess) r = block(i, false, down);
        if (r == cudaSuccess && tip_pending) r = tip(false, down);
        pending.clear();
        tip_pending = false;
        return r;
    }
    // Block i is final once the launches enqueued so far on s have run.
    cudaError_t give(int64_t i, cudaStream_t s) override {
        pending.push_back(i);
        return (int64_t)pending.size() >= kLinkGroup ? flush(s) : cudaSuccess;
    }
    // the whole matrix is resident: nothing to free
    cudaError_t release(int64_t, cudaStream_t) override { return cudaSuccess; }
    cudaError_t give_tip() override {
        tip_pending = true;
        return cudaSuccess;
    }
    // The remaining downloads, then s waits for them.
    cudaError_t finish(cudaStream_t s) override {
        cudaError_t r = flush(s);
        cudaEvent_t e;
        if (r == cudaSuccess) r = event(&e);
        if (r == cudaSuccess) r = cudaEventRecord(e, down);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(s, e, 0);
        return r;
    }
    ~HostLink() override {
        // released once their pending work completes
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        if (up) cudaStreamDestroy(up);
        if (down) cudaStreamDestroy(down);
    }
};

// Host-resident stacks streamed through a ring of R device slots, for
// matrices of any size (the reference's device_streaming, pobtaf.py:284-524,
// pobtasi.py:247-496, double-buffers two blocks; here R slots).  Block i
// lives in slot (i - off) mod R while the sweep needs it.  In sweep order
// (ascending for pobtaf, descending for pobtasi) block q's slot was last
// held by the block R positions earlier: its upload (copy stream `up`)
// waits until that block was released by the sweep and downloaded (copy
// stream `down`); uploads run ahead of the sweep as far as slots allow.
// The tip stays on the device for the whole call.
struct HostRing : Link {
    const sgb_bta* h = nullptr;  // host stacks
    char* dD = nullptr;          // ring slots: D, Lo, Ar of R blocks
    char* dLo = nullptr;
    char* dAr = nullptr;
    char* dT = nullptr;          // device tip
    int64_t R = 0, off = 0;
    bool ascending = true;
    size_t es = 8;
    cudaStream_t up = nullptr, down = nullptr;
    std::vector<cudaEvent_t> up_ev, freed, events;
    std::vector<char> released;
    int64_t next_up = 0;
    bool tip_final = false;

    int64_t blk(int64_t q) const { return ascending ? q : h->n - 1 - q; }
    int64_t pos(int64_t i) const { return ascending ? i : h->n - 1 - i; }
    int64_t slot(int64_t i) const {
        const int64_t r = (i - off) % R;
        return r < 0 ? r + R : r;
    }
    cudaError_t event(cudaEvent_t* e) {
        cudaError_t r = cudaEventCreateWithFlags(e, cudaEventDisableTiming);
        if (r == cudaSuccess) events.push_back(*e);
        return r;
    }
    cudaError_t copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st) {
        return bytes ? cudaMemcpyAsync(dst, src, bytes, kind, st) : cudaSuccess;
    }
    cudaError_t move(int64_t i, bool to_dev, cudaStream_t st) {
        const int64_t n = h->n, b = h->b, a = h->a, sl = slot(i);
        const cudaMemcpyKind k = to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
        auto mv = [&](void* hb, char* db, int64_t hoff, int64_t doff, int64_t cnt) {
            char* hp = (char*)hb + es * hoff;
            char* dp = db + es * doff;
            return to_dev ? copy(dp, hp, es * cnt, k, st) : copy(hp, dp, es * cnt, k, st);
        };
        cudaError_t r = mv(h->diag, dD, i * b * b, sl * b * b, b * b);
        if (r == cudaSuccess && i < n - 1) r = mv(h->lower, dLo, i * b * b, sl * b * b, b * b);
        if (r == cudaSuccess && a) r = mv(h->arrow, dAr, i * a * b, sl * a * b, a * b);
        return r;
    }
    // Enqueue the uploads whose slots are free, in sweep order.
    cudaError_t pump() {
        const int64_t n = h->n;
        while (next_up < n) {
            const int64_t q = next_up;
            if (q >= R && !released[(size_t)(q - R)]) break;
            const int64_t i = blk(q), sl = slot(i);
            cudaError_t r = cudaSuccess;
            if (q >= R) r = cudaStreamWaitEvent(up, freed[(size_t)sl], 0);
            if (r == cudaSuccess) r = move(i, true, up);
            if (r == cudaSuccess) r = cudaEventRecord(up_ev[(size_t)sl], up);
            if (r != cudaSuccess) return r;
            ++next_up;
        }
        return cudaSuccess;
    }
    cudaError_t start(cudaStream_t s) override {
        const int64_t n = h->n, a = h->a;
        released.assign((size_t)n, 0);
        up_ev.resize((size_t)R);
        freed.resize((size_t)R);
        cudaError_t r = cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking);
        if (r == cudaSuccess) r = cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking);
        for (int64_t k = 0; k < R && r == cudaSuccess; ++k) {
            r = event(&up_ev[(size_t)k]);
            if (r == cudaSuccess) r = event(&freed[(size_t)k]);
        }
        cudaEvent_t e0, et;
        if (r == cudaSuccess) r = event(&e0);
        if (r == cudaSuccess) r = cudaEventRecord(e0, s);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(up, e0, 0);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(down, e0, 0);
        if (r == cudaSuccess && a) r = copy(dT, h->tip, es * a * a, cudaMemcpyHostToDevice, up);
        if (r == cudaSuccess) r = event(&et);
        if (r == cudaSuccess) r = cudaEventRecord(et, up);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(s, et, 0);
        if (r == cudaSuccess) r = pump();
        return r;
    }
    cudaError_t need(int64_t i, cudaStream_t s) override {
        const int64_t q = pos(i);
        cudaError_t r = pump();
        if (r != cudaSuccess) return r;
        if (next_up <= q) return cudaErrorInvalidValue;  // ring too small for the sweep
        return cudaStreamWaitEvent(s, up_ev[(size_t)slot(i)], 0);
    }
    // final values leave when the slot is released
    cudaError_t give(int64_t, cudaStream_t) override { return cudaSuccess; }
    cudaError_t release(int64_t i, cudaStream_t s) override {
        const int64_t q = pos(i);
        if (released[(size_t)q]) return cudaSuccess;
        cudaEvent_t e;
        cudaError_t r = event(&e);
        if (r == cudaSuccess) r = cudaEventRecord(e, s);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(down, e, 0);
        if (r == cudaSuccess) r = move(i, false, down);
        if (r == cudaSuccess) r = cudaEventRecord(freed[(size_t)slot(i)], down);
        if (r != cudaSuccess) return r;
        released[(size_t)q] = 1;
        return pump();
    }
    cudaError_t give_tip() override {
        tip_final = true;
        return cudaSuccess;
    }
    cudaError_t finish(cudaStream_t s) override {
        cudaEvent_t e, d;
        cudaError_t r = event(&e);
        if (r == cudaSuccess) r = cudaEventRecord(e, s);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(down, e, 0);
        if (r == cudaSuccess && h->a) r = copy(h->tip, dT, es * h->a * h->a, cudaMemcpyDeviceToHost, down);
        if (r == cudaSuccess) r = event(&d);
        if (r == cudaSuccess) r = cudaEventRecord(d, down);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(s, d, 0);
        return r;
    }
    ~HostRing() override {
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        if (up) cudaStreamDestroy(up);
        if (down) cudaStreamDestroy(down);
    }
};

// ---- pobtaf -------------------------------------------------------------
// Block Cholesky, src/serinv/algs/pobtaf.py:97-183.  Per block i:
//   [D_i; Lo_i; Ar_i] <- blocked Cholesky of the column block  (:117-139)
//   D_{i+1} -= Lo_i Lo_i^T, Ar_{i+1} -= Ar_i Lo_i^T, T -= Ar_i Ar_i^T  (:143-159)
template <typename T>
int pobtaf_run(const sgb_bta* m, int factorize_last_block, int S, int Si, void* ws, int32_t* info, cudaStream_t s,
               Link* hl = nullptr, T* xall = nullptr, bool* xall_filled = nullptr, int64_t ring = 0) {
    const int64_t n = m->n, b = m->b, a = m->a;
    T* Tp = (T*)m->tip;
    Blocks<T> B;
    B.D = (T*)m->diag;
    B.Lo = (T*)m->lower;
    B.Ar = (T*)m->arrow;
    B.bb = b * b;
    B.ab = a * b;
    B.R = ring;
    PobtafWs<T> L(m, S, Si);
    T* tinv = (T*)((char*)ws + L.tinv);
    Ctx cx;
    cx.slices = S;
    cx.tc = (char*)ws + L.tc;
    cx.tc_bytes = L.tc_bytes;
    cx.status = (int32_t*)((char*)ws + L.status);
    Ctx cxi = cx;  // products with L_ii^{-T}
    cxi.slices = Si ? Si : S;
    const int64_t bb = b * b, ab = a * b;
    T* Xinv0 = (T*)((char*)ws + L.xinv);

    // [D_i; rows below] <- Cholesky of the column block.  Native: one
    // blocked sweep over the tall column block (the TRSMs fold into the
    // rank-32 updates).  Mixed: the persistent launch factors D_i alone and
    // forms L_ii^{-T} on the FP64 pipe; the rows below become one
    // tensor-core product rows * L_ii^{-T}.
    unsigned* bar = (unsigned*)((char*)ws + L.bar);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    SGB_TRY(cudaStreamIsCapturing(s, &cap));
    // one cooperative launch per block (on part of the GPU when captured
    // into a graph beside other work, if the capturing thread allows it);
    // small blocks, and captures that do not, use the launch-based sweep.
    // In a batch graph the one launch per block also beats the ~25 launches
    // of an FP32 block's tile sweep (measured on the uneven batch: 4.5 %)
    const bool captured = cap != cudaStreamCaptureStatusNone;
    const int pgrid = captured ? capture_panel_grid() : 0;
    const bool persistent = (!captured || pgrid > 0) && b > 2 * kTile;
    // 7 slices is the accuracy mode: its TRSMs stay FP64 substitutions (the
    // product with L_ii^{-T} carries kappa(L_ii) times the slice truncation)
    bool mixed_inverse = S != 0 && (S < 7 || Si != 0) && persistent;
    // the launch writes only the upper block triangle of L_ii^{-T}
    // xall (n b x b blocks): keep every L_ii^{-T} for later sweeps on this factor
    if (mixed_inverse) SGB_TRY(cudaMemsetAsync(xall ? xall : Xinv0, 0, sizeof(T) * bb * (xall ? n : 1), s));
    auto factor = [&](int64_t i, RowSet<T> r1, RowSet<T> r2) -> int {
        T* Di = B.d(i);
        T* Xinv = xall ? xall + i * bb : Xinv0;
        if (mixed_inverse) {
            RowSet<T> none{nullptr, 0, b};
            cudaError_t e =
                factor_panel_persistent<T>(Di, b, b, none, none, tinv, bar, cx.status, info, i * b, s, Xinv, pgrid);
            if (e == cudaSuccess) {
                GemmProb<T> pr[2];
                int np = 0;
                for (RowSet<T> r : {r1, r2}) {
                    if (r.rows <= 0) continue;
                    GemmProb<T> p = prob<T>();  // rows <- rows * L_ii^{-T}, in place (operands are sliced first)
                    p.M = (int32_t)r.rows;
                    p.N = (int32_t)b;
                    set_term<T>(p, 0, r.p, r.ld, 0, Xinv, b, 0, b, KM_LT_N1);
                    p.Cout = r.p;
                    p.ldc = r.ld;
                    pr[np++] = p;
                }
                if (np) SGB_TRY(run_gemm<T>(cxi, pr, np, s));
                return SGB_OK;
            }
            if (e != cudaErrorNotSupported) return cuda_fail(e);
            mixed_inverse = false;  // too few SMs for the persistent launch
        }
        cudaError_t e = persistent ? factor_panel_persistent<T>(Di, b, b, r1, r2, tinv, bar, cx.status, info, i * b,
                                                                s, nullptr, pgrid)
                                   : cudaErrorNotSupported;
        if (e == cudaErrorNotSupported) e = factor_column_block<T>(Di, b, b, r1, r2, tinv, info, i * b, s);
        return e == cudaSuccess ? SGB_OK : cuda_fail(e);
    };

    if (hl) SGB_TRY(hl->start(s));
    for (int64_t i = 0; i < n - 1; ++i) {
        if (hl) SGB_TRY(hl->need(i, s));
        RowSet<T> r1{B.lo(i), b, b};
        RowSet<T> r2{a ? B.ar(i) : nullptr, a, b};
        int rc = factor(i, r1, r2);
        if (rc != SGB_OK) return rc;
        if (hl) SGB_TRY(hl->give(i, s));
        if (hl) SGB_TRY(hl->need(i + 1, s));

        const bool next_factored = (i + 1 < n - 1) || factorize_last_block;
        GemmProb<T> pr[3];
        int np = 0;
        {   // D_{i+1} -= Lo_i Lo_i^T
            GemmProb<T> p = prob<T>();
            p.M = p.N = (int32_t)b;
            set_term<T>(p, 0, B.lo(i), b, 0, B.lo(i), b, 1, b);
            p.alpha = T(-1);
            p.beta = T(1);
            p.Cin = p.Cout = B.d(i + 1);
            p.ldcin = p.ldc = b;
            p.lower_only = next_factored ? 1 : 0;
            pr[np++] = p;
        }
        if (a) {
            GemmProb<T> p = prob<T>();  // Ar_{i+1} -= Ar_i Lo_i^T
            p.M = (int32_t)a;
            p.N = (int32_t)b;
            set_term<T>(p, 0, B.ar(i), b, 0, B.lo(i), b, 1, b);
            p.alpha = T(-1);
            p.beta = T(1);
            p.Cin = p.Cout = B.ar(i + 1);
            p.ldcin = p.ldc = b;
            pr[np++] = p;
            GemmProb<T> q = prob<T>();  // T -= Ar_i Ar_i^T
            q.M = q.N = (int32_t)a;
            set_term<T>(q, 0, B.ar(i), b, 0, B.ar(i), b, 1, b);
            q.alpha = T(-1);
            q.beta = T(1);
            q.Cin = q.Cout = Tp;
            q.ldcin = q.ldc = a;
            q.lower_only = factorize_last_block ? 1 : 0;
            pr[np++] = q;
        }
        SGB_TRY(run_gemm<T>(cx, pr, np, s));
        if (hl) SGB_TRY(hl->release(i, s));  // block i is not read again
    }

    if (hl) SGB_TRY(hl->need(n - 1, s));
    if (factorize_last_block) {
        const int64_t i = n - 1;
        RowSet<T> r1{nullptr, 0, b};
        RowSet<T> r2{a ? B.ar(i) : nullptr, a, b};
        int rc = factor(i, r1, r2);
        if (rc != SGB_OK) return rc;
        if (a) {
            GemmProb<T> q = prob<T>();  // T -= Ar_{n-1} Ar_{n-1}^T  (:177-180)
            q.M = q.N = (int32_t)a;
            set_term<T>(q, 0, B.ar(i), b, 0, B.ar(i), b, 1, b);
            q.alpha = T(-1);
            q.beta = T(1);
            q.Cin = q.Cout = Tp;
            q.ldcin = q.ldc = a;
            q.lower_only = 1;
            SGB_TRY(run_gemm<T>(cx, &q, 1, s));
            RowSet<T> none{nullptr, 0, a};
            rc = (int)factor_column_block<T>(Tp, a, a, none, none, tinv, info, n * b, s);  // :183
            if (rc != cudaSuccess) return cuda_fail((cudaError_t)rc);
        }
    }
    if (hl) {
        SGB_TRY(hl->give(n - 1, s));
        SGB_TRY(hl->release(n - 1, s));
        SGB_TRY(hl->give_tip());
        SGB_TRY(hl->finish(s));
    }
    if (xall_filled) *xall_filled = xall != nullptr && mixed_inverse && factorize_last_block;
    return SGB_OK;
}

// ---- pobtasi ------------------------------------------------------------
// Selected inversion, src/serinv/algs/pobtasi.py:92-172.  All L_ii^{-1} are
// independent of the back-sweep, so they are formed up front in one batched
// triangular inversion.  Per block i (from the last one):
//   U = -X_D[i+1] Lo_i - X_A[i+1]^T Ar_i ;  V = -X_A[i+1] Lo_i - X_T Ar_i    (:153-163)
//   X_Lo = U L_ii^{-1} ; X_A = V L_ii^{-1}
//   X_D  = (L_ii^{-T} - X_Lo^T Lo_i - X_A^T Ar_i) L_ii^{-1}                  (:167-172)
// The last block (:114-139) is the same step without the i+1 terms.
// Selected inversion, src/serinv/algs/pobtasi.py:92-172, rearranged so that
// the back-sweep chain is two grouped products per block.  With
// G_i = Lo_i L_ii^{-1}, H_i = Ar_i L_ii^{-1}, P_i = L_ii^{-T} L_ii^{-1}
// (batched over a chunk of blocks, off the chain) the reference's updates
// (:150-169) read
//   [X_{i+1,i}; X_{A,i}] = -[X_{i+1,i+1} X_{A,i+1}^T; X_{A,i+1} X_T] [G_i; H_i]
//   X_{i,i}              = P_i - X_{i+1,i}^T G_i - X_{A,i}^T H_i
// and the last block (:121-137) is the same without the i+1 terms.  L_ii,
// Lo_i and Ar_i are dead once G_i, H_i, P_i exist, so P_i is formed in the
// diagonal block itself and the outputs overwrite the factor in place.
template <typename T>
int pobtasi_run(const sgb_bta* m, int invert_last_block, int S, int Si, void* ws, cudaStream_t s,
                Link* hl = nullptr, const T* xall = nullptr, int64_t ring = 0) {
    const int64_t n = m->n, b = m->b, a = m->a;
    T* Tp = (T*)m->tip;
    // a ring holds two chunks: the one being swept and the one above it
    PobtasiWs<T> W(m, S, Si, ring ? ring / 2 : kSiChunk);
    Blocks<T> B;
    B.D = (T*)m->diag;
    B.Lo = (T*)m->lower;
    B.Ar = (T*)m->arrow;
    B.bb = b * b;
    B.ab = a * b;
    B.R = ring;
    B.off = invert_last_block ? n : n - 1;  // chunks end at multiples of the chunk size from here
    char* base = (char*)ws;
    Ctx cx;
    cx.slices = S;
    cx.tc = base + W.tc;
    cx.tc_bytes = W.tc_bytes;
    cx.status = (int32_t*)(base + W.status);
    Ctx cxi = cx;  // the inversions and the products with L_ii^{-1}
    cxi.slices = Si ? Si : S;
    T* Linv = (T*)(base + W.linv);
    T* Ltinv = (T*)(base + W.linv_tip);
    T* trs = (T*)(base + W.trtri);
    T* GH = (T*)(base + W.gh);
    const int64_t bb = b * b, ab = a * b, ghs = (b + a) * b;

    if (hl) {
        SGB_TRY(hl->start(s));
        SGB_TRY(hl->need(n - 1, s));
    }
    if (invert_last_block && a) {
        // X_T = L_T^{-T} L_T^{-1}  (:115-119)
        SGB_TRY(trtri_run<T>(cxi, Tp, a, 1, Ltinv, trs, s));
        GemmProb<T> p = prob<T>();
        p.M = p.N = (int32_t)a;
        set_term<T>(p, 0, Ltinv, a, 1, Ltinv, a, 0, a, KM_GE_M0);
        p.Cout = Tp;
        p.ldc = a;
        SGB_TRY(run_gemm<T>(cxi, &p, 1, s));
    }
    if (hl) SGB_TRY(hl->give_tip());

    // blocks whose L_ii is inverted here: all, or all but the last
    const int64_t ninv = invert_last_block ? n : n - 1;
    const int64_t tcb = S ? (W.chunk < kSiTcBatch ? W.chunk : kSiTcBatch) : W.chunk;
    for (int64_t hi = ninv; hi > 0; hi -= W.chunk) {
        const int64_t lo = hi > W.chunk ? hi - W.chunk : 0;
        if (hl) SGB_TRY(hl->need(lo, s));
        if (!B.contiguous(lo, hi)) return SGB_ERR_WORKSPACE;
        // with xall the inverses exist already, as L_jj^{-T}: operands are read transposed
        if (!xall) SGB_TRY(trtri_run<T>(cxi, B.d(lo), b, hi - lo, Linv, trs, s));
        for (int64_t j0 = lo; j0 < hi; j0 += tcb) {
            const int64_t jn = (hi - j0) < tcb ? (hi - j0) : tcb;
            const int64_t ng = (j0 + jn <= n - 1) ? jn : (n - 1 - j0);  // blocks with a Lo_j
            const T* Lj = xall ? xall + j0 * bb : Linv + (j0 - lo) * bb;
            const int tl = xall ? 1 : 0;  // L_jj^{-1} = op(Lj)
            T* GHj = GH + (j0 - lo) * ghs;
            GemmProb<T> pr[3];
            int np = 0;
            if (ng > 0) {  // G_j = Lo_j L_jj^{-1}
                GemmProb<T> p = prob<T>();
                p.M = p.N = (int32_t)b;
                p.batch = (int32_t)ng;
                set_term<T>(p, 0, B.lo(j0), b, 0, Lj, b, tl, b, KM_GE_N0);
                p.term[0].strideA = bb;
                p.term[0].strideB = bb;
                p.Cout = GHj;
                p.ldc = b;
                p.strideC = ghs;
                pr[np++] = p;
            }
            if (a) {  // H_j = Ar_j L_jj^{-1}
                GemmProb<T> p = prob<T>();
                p.M = (int32_t)a;
                p.N = (int32_t)b;
                p.batch = (int32_t)jn;
                set_term<T>(p, 0, B.ar(j0), b, 0, Lj, b, tl, b, KM_GE_N0);
                p.term[0].strideA = ab;
                p.term[0].strideB = bb;
                p.Cout = GHj + bb;
                p.ldc = b;
                p.strideC = ghs;
                pr[np++] = p;
            }
            {  // P_j = L_jj^{-T} L_jj^{-1} into D_j
                GemmProb<T> p = prob<T>();
                p.M = p.N = (int32_t)b;
                p.batch = (int32_t)jn;
                set_term<T>(p, 0, Lj, b, 1 - tl, Lj, b, tl, b, KM_GE_M0);
                p.term[0].strideA = bb;
                p.term[0].strideB = bb;
                p.Cout = B.d(j0);
                p.ldc = b;
                p.strideC = bb;
                pr[np++] = p;
            }
            SGB_TRY(run_gemm<T>(cxi, pr, np, s));
        }
        for (int64_t i = hi - 1; i >= lo; --i) {
            const bool has_next = i < n - 1;
            const T* G = GH + (i - lo) * ghs;
            const T* H = G + bb;
            GemmProb<T> pr[2];
            int np = 0;
            if (has_next) {  // X_{i+1,i} = -(X_{i+1,i+1} G_i + X_{A,i+1}^T H_i)  (:150-155)
                GemmProb<T> p = prob<T>();
                p.M = p.N = (int32_t)b;
                set_term<T>(p, 0, B.d(i + 1), b, 0, G, b, 0, b);
                if (a) set_term<T>(p, 1, B.ar(i + 1), b, 1, H, b, 0, a);
                p.alpha = T(-1);
                p.Cout = B.lo(i);
                p.ldc = b;
                pr[np++] = p;
            }
            if (a) {  // X_{A,i} = -(X_{A,i+1} G_i + X_T H_i)  (:157-162, :128-130)
                GemmProb<T> p = prob<T>();
                p.M = (int32_t)a;
                p.N = (int32_t)b;
                int t = 0;
                if (has_next) set_term<T>(p, t++, B.ar(i + 1), b, 0, G, b, 0, b);
                set_term<T>(p, t, Tp, a, 0, H, b, 0, a);
                p.alpha = T(-1);
                p.Cout = B.ar(i);
                p.ldc = b;
                pr[np++] = p;
            }
            if (np > 0) {  // (a == 0 and no next block: X_ii = P_i)
                SGB_TRY(run_gemm<T>(cx, pr, np, s));
                // X_ii = P_i - X_{i+1,i}^T G_i - X_{A,i}^T H_i  (:164-169, :133-137)
                GemmProb<T> p = prob<T>();
                p.M = p.N = (int32_t)b;
                int t = 0;
                if (has_next) set_term<T>(p, t++, B.lo(i), b, 1, G, b, 0, b);
                if (a) set_term<T>(p, t++, B.ar(i), b, 1, H, b, 0, a);
                p.alpha = T(-1);
                p.beta = T(1);
                p.Cin = B.d(i);
                p.ldcin = b;
                p.Cout = B.d(i);
                p.ldc = b;
                SGB_TRY(run_gemm<T>(cx, &p, 1, s));
            }
            if (hl) {
                SGB_TRY(hl->give(i, s));
                if (has_next) SGB_TRY(hl->release(i + 1, s));  // block i+1 was read for the last time
            }
        }
    }
    if (hl) {
        if (!invert_last_block) SGB_TRY(hl->give(n - 1, s));
        SGB_TRY(hl->release(0, s));
        SGB_TRY(hl->finish(s));
    }
    return SGB_OK;
}

// ---- pobtas -------------------------------------------------------------
// Block triangular solve, src/serinv/algs/pobtas.py:65-161.  The diagonal
// solves use L_ii^{-1} (one batched triangular inversion up front), so every
// block step is two grouped products.
template <typename T>
int pobtas_native(const sgb_bta* m, T* Bm, int64_t nrhs, int64_t ldb, char trans, int partial, void* ws,
                  cudaStream_t s, bool have_linv = false, const T* xall = nullptr) {
    const int64_t n = m->n, b = m->b, a = m->a;
    T* D = (T*)m->diag;
    T* Lo = (T*)m->lower;
    T* Ar = (T*)m->arrow;
    T* Tp = (T*)m->tip;
    PobtasWs<T> W(m, nrhs);
    char* base = (char*)ws;
    T* Linv = (T*)(base + W.linv);
    T* Ltinv = (T*)(base + W.linv_tip);
    T* trs = (T*)(base + W.trtri);
    T* y = (T*)(base + W.y);
    const int64_t bb = b * b, ab = a * b;
    T* Btip = Bm + n * b * ldb;
    auto Bi = [&](int64_t i) { return Bm + i * b * ldb; };

    if (nrhs == 0) return SGB_OK;
    Ctx native;
    // have_linv: the workspace holds the inverses from an earlier call with this factor
    if (!have_linv) {
        // with xall the block inverses exist already, as L_ii^{-T} (read transposed)
        if (!xall) SGB_TRY(trtri_run<T>(native, D, b, n, Linv, trs, s));
        if (a && !partial) SGB_TRY(trtri_run<T>(native, Tp, a, 1, Ltinv, trs, s));
    }
    const T* Li = xall ? xall : Linv;
    const int tl = xall ? 1 : 0;

    if (trans == 'N') {
        const int64_t last = partial ? n - 1 : n;
        for (int64_t i = 0; i < last; ++i) {
            // y = L_ii^{-1} B_i
            GemmProb<T> p = prob<T>();
            p.M = (int32_t)b;
            p.N = (int32_t)nrhs;
            set_term<T>(p, 0, Li + i * bb, b, tl, Bi(i), ldb, 0, b, KM_LT_M1);
            p.Cout = y;
            p.ldc = nrhs;
            SGB_TRY(gemm_simt<T>(&p, 1, s));
            // B_i = y ; B_{i+1} -= Lo_i y ; B_tip -= Ar_i y
            GemmProb<T> pr[3];
            int np = 0;
            pr[np++] = copy_prob<T>(Bi(i), ldb, y, nrhs, b, nrhs);
            if (i < n - 1) {
                GemmProb<T> q = prob<T>();
                q.M = (int32_t)b;
                q.N = (int32_t)nrhs;
                set_term<T>(q, 0, Lo + i * bb, b, 0, y, nrhs, 0, b);
                q.alpha = T(-1);
                q.beta = T(1);
                q.Cin = q.Cout = Bi(i + 1);
                q.ldcin = q.ldc = ldb;
                pr[np++] = q;
            }
            if (a) {
                GemmProb<T> q = prob<T>();
                q.M = (int32_t)a;
                q.N = (int32_t)nrhs;
                set_term<T>(q, 0, Ar + i * ab, b, 0, y, nrhs, 0, b);
                q.alpha = T(-1);
                q.beta = T(1);
                q.Cin = q.Cout = Btip;
                q.ldcin = q.ldc = ldb;
                pr[np++] = q;
            }
            SGB_TRY(gemm_simt<T>(pr, np, s));
        }
        if (!partial && a) {
            // B_tip = L_T^{-1} B_tip  (:124-126)
            GemmProb<T> p = prob<T>();
            p.M = (int32_t)a;
            p.N = (int32_t)nrhs;
            set_term<T>(p, 0, Ltinv, a, 0, Btip, ldb, 0, a, KM_LT_M1);
            p.Cout = y;
            p.ldc = nrhs;
            SGB_TRY(gemm_simt<T>(&p, 1, s));
            GemmProb<T> c = copy_prob<T>(Btip, ldb, y, nrhs, a, nrhs);
            SGB_TRY(gemm_simt<T>(&c, 1, s));
        }
        return SGB_OK;
    }

    // trans 'T' / 'C' (real arithmetic: identical)
    if (!partial) {
        if (a) {
            // B_tip = L_T^{-T} B_tip  (:131-136)
            GemmProb<T> p = prob<T>();
            p.M = (int32_t)a;
            p.N = (int32_t)nrhs;
            set_term<T>(p, 0, Ltinv, a, 1, Btip, ldb, 0, a, KM_GE_M0);
            p.Cout = y;
            p.ldc = nrhs;
            SGB_TRY(gemm_simt<T>(&p, 1, s));
            GemmProb<T> c = copy_prob<T>(Btip, ldb, y, nrhs, a, nrhs);
            SGB_TRY(gemm_simt<T>(&c, 1, s));
        }
    }
    const int64_t first = partial ? n - 2 : n - 1;
    for (int64_t i = first; i >= 0; --i) {
        // B_i -= Lo_i^T B_{i+1} + Ar_i^T B_tip  (:139-159)
        GemmProb<T> p = prob<T>();
        p.M = (int32_t)b;
        p.N = (int32_t)nrhs;
        int t = 0;
        if (i < n - 1) set_term<T>(p, t++, Lo + i * bb, b, 1, Bi(i + 1), ldb, 0, b);
        if (a) set_term<T>(p, t++, Ar + i * ab, b, 1, Btip, ldb, 0, a);
        if (t) {
            p.alpha = T(-1);
            p.beta = T(1);
            p.Cin = p.Cout = Bi(i);
            p.ldcin = p.ldc = ldb;
            SGB_TRY(gemm_simt<T>(&p, 1, s));
        }
        // B_i = L_ii^{-T} B_i
        GemmProb<T> q = prob<T>();
        q.M = (int32_t)b;
        q.N = (int32_t)nrhs;
        set_term<T>(q, 0, Li + i * bb, b, 1 - tl, Bi(i), ldb, 0, b, KM_GE_M0);
        q.Cout = y;
        q.ldc = nrhs;
        SGB_TRY(gemm_simt<T>(&q, 1, s));
        GemmProb<T> c = copy_prob<T>(Bi(i), ldb, y, nrhs, b, nrhs);
        SGB_TRY(gemm_simt<T>(&c, 1, s));
    }
    return SGB_OK;
}

// ---- permuted (middle-partition) variants -------------------------------
// The two-sided elimination of a middle partition with the fill-in column
// `buf` (n, b, b): buf[i] holds the top block row's coupling to block i
// (src/serinv/algs/pobtaf.py:186-281, pobtasi.py:175-244, pobtas.py:
// 164-218).  Storage precision only (SIMT products, launch-based tile
// sweep); the reduced system (blocks 0 and n-1, the tip) is the caller's.

template <typename T>
GemmProb<T> upd_prob(T* C, int64_t ldc, int64_t M, int64_t N, T alpha, T beta) {
    GemmProb<T> p = prob<T>();
    p.M = (int32_t)M;
    p.N = (int32_t)N;
    p.alpha = alpha;
    p.beta = beta;
    if (beta != T(0)) {
        p.Cin = C;
        p.ldcin = ldc;
    }
    p.Cout = C;
    p.ldc = ldc;
    return p;
}

template <typename T>
int pobtaf_permuted_run(const sgb_bta* m, T* buf, int S, int Si, void* ws, int32_t* info, cudaStream_t s) {
    const int64_t n = m->n, b = m->b, a = m->a;
    T* D = (T*)m->diag;
    T* Lo = (T*)m->lower;
    T* Ar = (T*)m->arrow;
    T* Tp = (T*)m->tip;
    PobtafWs<T> L(m, S, Si);
    T* tinv = (T*)((char*)ws + L.tinv);
    Ctx cx;
    cx.slices = S;
    cx.tc = (char*)ws + L.tc;
    cx.tc_bytes = L.tc_bytes;
    cx.status = (int32_t*)((char*)ws + L.status);
    Ctx cxi = cx;
    cxi.slices = Si ? Si : S;
    unsigned* bar = (unsigned*)((char*)ws + L.bar);
    T* Xinv = (T*)((char*)ws + L.xinv);
    const int64_t bb = b * b, ab = a * b;
    // mixed: the persistent column-block kernel factors D_i and forms
    // L_ii^{-T}; the three row sets below become one tensor-core product
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    SGB_TRY(cudaStreamIsCapturing(s, &cap));
    bool mixed_inverse = S != 0 && (S < 7 || Si != 0) && b > 2 * kTile && cap == cudaStreamCaptureStatusNone;
    if (mixed_inverse) SGB_TRY(cudaMemsetAsync(Xinv, 0, sizeof(T) * bb, s));
    {   // buf[1] = Lo[0]^T  (pobtaf.py:203)
        GemmProb<T> c = copy_prob<T>(buf + bb, b, Lo, b, b, b);
        c.transCin = 1;
        SGB_TRY(gemm_simt<T>(&c, 1, s));
    }
    for (int64_t i = 1; i < n - 1; ++i) {  // :206
        // [D_i; Lo_i; buf_i; Ar_i] <- Cholesky of the column block  (:208-242)
        RowSet<T> r1{Lo + i * bb, b, b}, r2{buf + i * bb, b, b}, r3{a ? Ar + i * ab : nullptr, a, b};
        bool done = false;
        if (mixed_inverse) {
            RowSet<T> none{nullptr, 0, b};
            cudaError_t e = factor_panel_persistent<T>(D + i * bb, b, b, none, none, tinv, bar, cx.status, info, i * b,
                                                       s, Xinv, 0);
            if (e == cudaSuccess) {
                GemmProb<T> pr[3];
                int np = 0;
                for (RowSet<T> r : {r1, r2, r3}) {
                    if (r.rows <= 0 || r.p == nullptr) continue;
                    GemmProb<T> p = prob<T>();  // rows <- rows * L_ii^{-T}, in place (operands are sliced first)
                    p.M = (int32_t)r.rows;
                    p.N = (int32_t)b;
                    set_term<T>(p, 0, r.p, r.ld, 0, Xinv, b, 0, b, KM_LT_N1);
                    p.Cout = r.p;
                    p.ldc = r.ld;
                    pr[np++] = p;
                }
                SGB_TRY(run_gemm<T>(cxi, pr, np, s));
                done = true;
            } else if (e != cudaErrorNotSupported) {
                return cuda_fail(e);
            } else {
                mixed_inverse = false;  // too few SMs for the persistent launch
            }
        }
        if (!done) {
            cudaError_t e = factor_column_block<T>(D + i * bb, b, b, r1, r2, tinv, info, i * b, s, r3);
            if (e != cudaSuccess) return cuda_fail(e);
        }
        GemmProb<T> pr[6];
        int np = 0;
        const T* lo = Lo + i * bb;
        const T* bu = buf + i * bb;
        const T* ar = Ar + i * ab;
        GemmProb<T> p = upd_prob<T>(D + (i + 1) * bb, b, b, b, T(-1), T(1));  // :246-250
        set_term<T>(p, 0, lo, b, 0, lo, b, 1, b);
        pr[np++] = p;
        p = upd_prob<T>(D, b, b, b, T(-1), T(1));  // D_0 -= buf_i buf_i^T  (:267-269)
        set_term<T>(p, 0, bu, b, 0, bu, b, 1, b);
        pr[np++] = p;
        p = upd_prob<T>(buf + (i + 1) * bb, b, b, b, T(-1), T(0));  // buf_{i+1} = -buf_i Lo_i^T  (:272-274)
        set_term<T>(p, 0, bu, b, 0, lo, b, 1, b);
        pr[np++] = p;
        if (a) {
            p = upd_prob<T>(Ar + (i + 1) * ab, b, a, b, T(-1), T(1));  // :253-256
            set_term<T>(p, 0, ar, b, 0, lo, b, 1, b);
            pr[np++] = p;
            p = upd_prob<T>(Tp, a, a, a, T(-1), T(1));  // :260-263
            set_term<T>(p, 0, ar, b, 0, ar, b, 1, b);
            pr[np++] = p;
            p = upd_prob<T>(Ar, b, a, b, T(-1), T(1));  // Ar_0 -= Ar_i buf_i^T  (:278-281)
            set_term<T>(p, 0, ar, b, 0, bu, b, 1, b);
            pr[np++] = p;
        }
        SGB_TRY(run_gemm_groups<T>(cx, pr, np, s));
    }
    return SGB_OK;
}

// pobtasi_permuted scratch: per chunk of blocks L_ii^{-1}, G_i = Lo_i L_ii^{-1},
// F_i = buf_i L_ii^{-1}, H_i = Ar_i L_ii^{-1}, and the inversion scratch.
template <typename T>
struct PobtasiPermWs {
    size_t status, linv, trtri, gfh, tc, tc_bytes, total;
    int64_t chunk;
    explicit PobtasiPermWs(const sgb_bta* m, int S = 0, int Si = 0) {
        const int64_t n = m->n, b = m->b, a = m->a;
        chunk = n < kSiChunk ? (n > 0 ? n : 1) : kSiChunk;
        Carve c;
        status = c.take(256);
        tc_bytes = 0;
        if (Si > S) S = Si;
        if (S) {  // slice scratch of the largest tensor-core launch
            const int64_t tb = chunk < kSiTcBatch ? chunk : kSiTcBatch;
            const int64_t mx = b > a ? b : a;
            size_t need[3];
            need[0] = 3 * tc_prob_bytes(S, b, b, b, tb) + tc_prob_bytes(S, a, b, b, tb);  // G, F, H, P
            need[1] = trtri_tc_bytes(S, b, chunk);
            need[2] = 3 * tc_prob_bytes(S, mx, b, kTcMaxK, 1);  // one round of the back-sweep products
            for (size_t v : need) tc_bytes = v > tc_bytes ? v : tc_bytes;
        }
        tc = c.take(tc_bytes);
        linv = c.take(sizeof(T) * (size_t)(chunk * b * b));
        trtri = c.take(sizeof(T) * trtri_scratch_elems(b, chunk));
        gfh = c.take(sizeof(T) * (size_t)(chunk * (2 * b + a) * b));
        total = c.off;
    }
};

template <typename T>
int pobtasi_permuted_run(const sgb_bta* m, T* buf, int S, int Si, void* ws, cudaStream_t s) {
    const int64_t n = m->n, b = m->b, a = m->a;
    T* D = (T*)m->diag;
    T* Lo = (T*)m->lower;
    T* Ar = (T*)m->arrow;
    T* Tp = (T*)m->tip;
    PobtasiPermWs<T> W(m, S, Si);
    char* base = (char*)ws;
    T* Linv = (T*)(base + W.linv);
    T* trs = (T*)(base + W.trtri);
    T* GFH = (T*)(base + W.gfh);
    const int64_t bb = b * b, ab = a * b, gs = (2 * b + a) * b;
    Ctx cx;  // native, or tensor-core slice products
    cx.slices = S;
    cx.tc = base + W.tc;
    cx.tc_bytes = W.tc_bytes;
    cx.status = (int32_t*)(base + W.status);
    Ctx cxi = cx;  // the inversions and the products with L_ii^{-1}
    cxi.slices = Si ? Si : S;
    // blocks n-2 .. 1, in chunks from the bottom (pobtasi.py:199)
    const int64_t tcb = S ? (W.chunk < kSiTcBatch ? W.chunk : kSiTcBatch) : W.chunk;
    for (int64_t hi = n - 1; hi > 1; hi -= W.chunk) {
        const int64_t lo = hi - W.chunk > 1 ? hi - W.chunk : 1;
        const int64_t cnt = hi - lo;
        SGB_TRY(trtri_run<T>(cxi, D + lo * bb, b, cnt, Linv, trs, s));
        // G, F, H from the factor, P = L^{-T} L^{-1} into D_j (L_jj is dead
        // then), tcb blocks per launch
        for (int64_t j0 = lo; j0 < hi; j0 += tcb) {
            const int64_t jn = (hi - j0) < tcb ? (hi - j0) : tcb;
            T* GFHj = GFH + (j0 - lo) * gs;
            const T* Lj = Linv + (j0 - lo) * bb;
            GemmProb<T> pr[4];
            int np = 0;
            GemmProb<T> p = prob<T>();
            p.M = p.N = (int32_t)b;
            p.batch = (int32_t)jn;
            set_term<T>(p, 0, Lo + j0 * bb, b, 0, Lj, b, 0, b, KM_GE_N0);
            p.term[0].strideA = bb;
            p.term[0].strideB = bb;
            p.Cout = GFHj;
            p.ldc = b;
            p.strideC = gs;
            pr[np++] = p;
            GemmProb<T> q = p;
            q.term[0].A = buf + j0 * bb;
            q.Cout = GFHj + bb;
            pr[np++] = q;
            if (a) {
                GemmProb<T> h = prob<T>();
                h.M = (int32_t)a;
                h.N = (int32_t)b;
                h.batch = (int32_t)jn;
                set_term<T>(h, 0, Ar + j0 * ab, b, 0, Lj, b, 0, b, KM_GE_N0);
                h.term[0].strideA = ab;
                h.term[0].strideB = bb;
                h.Cout = GFHj + 2 * bb;
                h.ldc = b;
                h.strideC = gs;
                pr[np++] = h;
            }
            GemmProb<T> pp = prob<T>();
            pp.M = pp.N = (int32_t)b;
            pp.batch = (int32_t)jn;
            set_term<T>(pp, 0, Lj, b, 1, Lj, b, 0, b, KM_GE_M0);
            pp.term[0].strideA = bb;
            pp.term[0].strideB = bb;
            pp.Cout = D + j0 * bb;
            pp.ldc = b;
            pp.strideC = bb;
            pr[np++] = pp;
            SGB_TRY(run_gemm_groups<T>(cxi, pr, np, s));
        }
        for (int64_t i = hi - 1; i >= lo; --i) {
            const T* G = GFH + (i - lo) * gs;
            const T* F = G + bb;
            const T* H = G + 2 * bb;
            GemmProb<T> x[3];
            // X_{i+1,i} = -(X_{top,i+1}^T F + X_{i+1,i+1} G + X_{A,i+1}^T H)  (:211-216)
            x[0] = upd_prob<T>(Lo + i * bb, b, b, b, T(-1), T(0));
            set_term<T>(x[0], 0, buf + (i + 1) * bb, b, 1, F, b, 0, b);
            set_term<T>(x[0], 1, D + (i + 1) * bb, b, 0, G, b, 0, b);
            if (a) set_term<T>(x[0], 2, Ar + (i + 1) * ab, b, 1, H, b, 0, a);
            // X_{top,i} = -(X_{top,i+1} G + X_{top,top} F + X_{A,top}^T H)  (:219-223)
            x[1] = upd_prob<T>(buf + i * bb, b, b, b, T(-1), T(0));
            set_term<T>(x[1], 0, buf + (i + 1) * bb, b, 0, G, b, 0, b);
            set_term<T>(x[1], 1, D, b, 0, F, b, 0, b);
            if (a) set_term<T>(x[1], 2, Ar, b, 1, H, b, 0, a);
            int nx = 2;
            if (a) {  // X_{A,i} = -(X_{A,i+1} G + X_{A,top} F + X_T H)  (:227-231)
                x[2] = upd_prob<T>(Ar + i * ab, b, a, b, T(-1), T(0));
                set_term<T>(x[2], 0, Ar + (i + 1) * ab, b, 0, G, b, 0, b);
                set_term<T>(x[2], 1, Ar, b, 0, F, b, 0, b);
                set_term<T>(x[2], 2, Tp, a, 0, H, b, 0, a);
                nx = 3;
            }
            SGB_TRY(run_gemm_groups<T>(cx, x, nx, s));
            // X_ii = P_i - X_{i+1,i}^T G - X_{top,i}^T F - X_{A,i}^T H  (:234-241)
            GemmProb<T> d = upd_prob<T>(D + i * bb, b, b, b, T(-1), T(1));
            set_term<T>(d, 0, Lo + i * bb, b, 1, G, b, 0, b);
            set_term<T>(d, 1, buf + i * bb, b, 1, F, b, 0, b);
            if (a) set_term<T>(d, 2, Ar + i * ab, b, 1, H, b, 0, a);
            SGB_TRY(run_gemm_groups<T>(cx, &d, 1, s));
        }
    }
    // X_{1,0} = X_{top,1}^T  (:244)
    GemmProb<T> c = copy_prob<T>(Lo, b, buf + bb, b, b, b);
    c.transCin = 1;
    SGB_TRY(gemm_simt<T>(&c, 1, s));
    return SGB_OK;
}

template <typename T>
int pobtas_permuted_run(const sgb_bta* m, T* buf, T* Bm, int64_t nrhs, int64_t ldb, char trans, void* ws,
                        cudaStream_t s) {
    const int64_t n = m->n, b = m->b, a = m->a;
    T* D = (T*)m->diag;
    T* Lo = (T*)m->lower;
    T* Ar = (T*)m->arrow;
    PobtasWs<T> W(m, nrhs);
    char* base = (char*)ws;
    T* Linv = (T*)(base + W.linv);
    T* trs = (T*)(base + W.trtri);
    T* y = (T*)(base + W.y);
    const int64_t bb = b * b, ab = a * b;
    T* Btip = Bm + n * b * ldb;
    auto Bi = [&](int64_t i) { return Bm + i * b * ldb; };
    if (nrhs == 0 || n < 3) return SGB_OK;
    Ctx native;
    SGB_TRY(trtri_run<T>(native, D + bb, b, n - 2, Linv, trs, s));  // blocks 1 .. n-2
    auto Li = [&](int64_t i) { return Linv + (i - 1) * bb; };
    if (trans == 'N') {  // pobtas.py:179-203
        for (int64_t i = 1; i < n - 1; ++i) {
            GemmProb<T> p = prob<T>();  // y = L_ii^{-1} B_i
            p.M = (int32_t)b;
            p.N = (int32_t)nrhs;
            set_term<T>(p, 0, Li(i), b, 0, Bi(i), ldb, 0, b, KM_LT_M1);
            p.Cout = y;
            p.ldc = nrhs;
            SGB_TRY(gemm_simt<T>(&p, 1, s));
            GemmProb<T> pr[4];
            int np = 0;
            pr[np++] = copy_prob<T>(Bi(i), ldb, y, nrhs, b, nrhs);
            GemmProb<T> q = upd_prob<T>(Bi(i + 1), ldb, b, nrhs, T(-1), T(1));
            set_term<T>(q, 0, Lo + i * bb, b, 0, y, nrhs, 0, b);
            pr[np++] = q;
            q = upd_prob<T>(Bi(0), ldb, b, nrhs, T(-1), T(1));
            set_term<T>(q, 0, buf + i * bb, b, 0, y, nrhs, 0, b);
            pr[np++] = q;
            if (a) {
                q = upd_prob<T>(Btip, ldb, a, nrhs, T(-1), T(1));
                set_term<T>(q, 0, Ar + i * ab, b, 0, y, nrhs, 0, b);
                pr[np++] = q;
            }
            SGB_TRY(gemm_simt<T>(pr, np, s));
        }
        return SGB_OK;
    }
    for (int64_t i = n - 2; i >= 1; --i) {  // pobtas.py:204-216
        GemmProb<T> p = upd_prob<T>(Bi(i), ldb, b, nrhs, T(-1), T(1));
        set_term<T>(p, 0, Lo + i * bb, b, 1, Bi(i + 1), ldb, 0, b);
        set_term<T>(p, 1, buf + i * bb, b, 1, Bi(0), ldb, 0, b);
        if (a) set_term<T>(p, 2, Ar + i * ab, b, 1, Btip, ldb, 0, a);
        SGB_TRY(gemm_simt<T>(&p, 1, s));
        GemmProb<T> q = prob<T>();  // y = L_ii^{-T} B_i
        q.M = (int32_t)b;
        q.N = (int32_t)nrhs;
        set_term<T>(q, 0, Li(i), b, 1, Bi(i), ldb, 0, b, KM_GE_M0);
        q.Cout = y;
        q.ldc = nrhs;
        SGB_TRY(gemm_simt<T>(&q, 1, s));
        GemmProb<T> c = copy_prob<T>(Bi(i), ldb, y, nrhs, b, nrhs);
        SGB_TRY(gemm_simt<T>(&c, 1, s));
    }
    return SGB_OK;
}

// ---- refined solve ---------------------------------------------------------
// x = A^{-1} B by the factor L, refined against the original A:
//   x <- L^{-T} L^{-1} B ; repeat: r = B - A x, x += L^{-T} L^{-1} r.
// The residual is formed in the storage precision from A's lower stacks;
// the block inverses of L are formed once and reused by every solve.
template <typename T>
struct RefineWs {
    size_t solve, x, r, total;
    RefineWs(const sgb_bta* L, int64_t nrhs) {
        const size_t N = (size_t)(L->n * L->b + L->a);
        Carve c;
        solve = c.take(PobtasWs<T>(L, nrhs).total);
        x = c.take(sizeof(T) * N * (size_t)nrhs);
        r = c.take(sizeof(T) * N * (size_t)nrhs);
        total = c.off;
    }
};

template <typename T>
int pobtas_refine_run(const sgb_bta* A, const sgb_bta* L, T* B, int64_t nrhs, int64_t ldb, int iters, void* ws,
                      cudaStream_t s) {
    if (nrhs == 0) return SGB_OK;
    RefineWs<T> W(L, nrhs);
    char* base = (char*)ws;
    void* sw = base + W.solve;
    T* x = (T*)(base + W.x);
    T* r = (T*)(base + W.r);
    const int64_t N = L->n * L->b + L->a;
    const size_t row = sizeof(T) * (size_t)nrhs;
    SGB_TRY(cudaMemcpy2DAsync(x, row, B, sizeof(T) * ldb, row, N, cudaMemcpyDeviceToDevice, s));
    int rc = pobtas_native<T>(L, x, nrhs, nrhs, 'N', 0, sw, s, false);
    if (rc == SGB_OK) rc = pobtas_native<T>(L, x, nrhs, nrhs, 'C', 0, sw, s, true);
    for (int k = 0; k < iters && rc == SGB_OK; ++k) {
        SGB_TRY(cudaMemcpy2DAsync(r, row, B, sizeof(T) * ldb, row, N, cudaMemcpyDeviceToDevice, s));
        SGB_TRY(bta_symv<T>(A, x, nrhs, r, nrhs, nrhs, T(-1), T(1), s));
        rc = pobtas_native<T>(L, r, nrhs, nrhs, 'N', 0, sw, s, true);
        if (rc == SGB_OK) rc = pobtas_native<T>(L, r, nrhs, nrhs, 'C', 0, sw, s, true);
        if (rc == SGB_OK) SGB_TRY(axpy2d<T>(x, nrhs, r, nrhs, N, nrhs, s));
    }
    if (rc != SGB_OK) return rc;
    SGB_TRY(cudaMemcpy2DAsync(B, sizeof(T) * ldb, x, row, row, N, cudaMemcpyDeviceToDevice, s));
    return SGB_OK;
}

// ---- batch plan items ------------------------------------------------------
// pobtaf -> pobtas (N, T) -> pobtasi of one matrix inside a batch plan.  In
// the mixed form with the persistent column-block kernel every L_ii^{-T} is
// formed by pobtaf anyway; the item keeps them (n b x b blocks at the front
// of its workspace) so that the solve and the selected inversion skip their
// batched triangular inversions.
bool item_keeps_inverses(const sgb_bta* m, int precision, int ops) {
    const int S = parse_precision(precision, m->dtype);
    return (ops & SGB_OP_POBTAF) && (ops & (SGB_OP_POBTAS | SGB_OP_POBTASI)) && m->dtype == SGB_F64 && S > 0 &&
           S < 7 && m->b > 2 * kTile && capture_panel_grid() > 0;
}

}  // namespace

size_t plan_item_ws(const sgb_bta* m, int ops, int precision, int64_t nrhs) {
    size_t need = 0, x = 0;
    if (ops & SGB_OP_POBTAF) {
        sgb_pobtaf_workspace_size(m, precision, &x);
        need = need > x ? need : x;
    }
    if (ops & SGB_OP_POBTASI) {
        sgb_pobtasi_workspace_size(m, precision, &x);
        need = need > x ? need : x;
    }
    if ((ops & SGB_OP_POBTAS) && nrhs > 0) {
        sgb_pobtas_workspace_size(m, nrhs, precision, &x);
        need = need > x ? need : x;
    }
    need = align_up(need);
    if (item_keeps_inverses(m, precision, ops)) need += align_up(sizeof(double) * (size_t)(m->n * m->b * m->b));
    return need;
}

int plan_item(const sgb_bta* m, int ops, int precision, void* rhs, int64_t nrhs, void* ws, size_t wsb,
              int32_t* info, cudaStream_t s) {
    if (!item_keeps_inverses(m, precision, ops)) {
        int rc = SGB_OK;
        if (ops & SGB_OP_POBTAF) rc = sgb_pobtaf(m, 1, precision, ws, wsb, info, s);
        if (rc == SGB_OK && (ops & SGB_OP_POBTAS) && nrhs > 0) {
            rc = sgb_pobtas(m, rhs, nrhs, nrhs, 'N', 0, precision, ws, wsb, s);
            if (rc == SGB_OK) rc = sgb_pobtas(m, rhs, nrhs, nrhs, 'T', 0, precision, ws, wsb, s);
        }
        if (rc == SGB_OK && (ops & SGB_OP_POBTASI)) rc = sgb_pobtasi(m, 1, precision, ws, wsb, s);
        return rc;
    }
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    const size_t xbytes = align_up(sizeof(double) * (size_t)(m->n * m->b * m->b));
    if (wsb < xbytes) return SGB_ERR_WORKSPACE;
    double* xall = (double*)ws;
    void* w = (char*)ws + xbytes;
    const size_t wb = wsb - xbytes;
    size_t need = 0;
    sgb_pobtaf_workspace_size(m, precision, &need);
    if ((rc = check_ws(w, wb, need))) return rc;
    if (info) SGB_TRY(cudaMemsetAsync(info, 0, sizeof(int32_t), s));
    SGB_TRY(cudaMemsetAsync(w, 0, sizeof(int32_t), s));  // status word
    bool filled = false;
    const int Si = parse_inv_slices(precision, S);
    if ((rc = pobtaf_run<double>(m, 1, S, Si, w, info, s, nullptr, xall, &filled))) return rc;
    const double* xa = filled ? xall : nullptr;
    if ((ops & SGB_OP_POBTAS) && nrhs > 0) {
        sgb_pobtas_workspace_size(m, nrhs, precision, &need);
        if ((rc = check_ws(w, wb, need))) return rc;
        rc = pobtas_native<double>(m, (double*)rhs, nrhs, nrhs, 'N', 0, w, s, false, xa);
        if (rc == SGB_OK) rc = pobtas_native<double>(m, (double*)rhs, nrhs, nrhs, 'T', 0, w, s, false, xa);
        if (rc) return rc;
    }
    if (ops & SGB_OP_POBTASI) {
        sgb_pobtasi_workspace_size(m, precision, &need);
        if ((rc = check_ws(w, wb, need))) return rc;
        rc = pobtasi_run<double>(m, 1, S, Si, w, s, nullptr, xa);
    }
    return rc;
}

namespace {

// ---- streamed host-resident stacks ----------------------------------------
// Workspace of sgb_pobtaf_stream / sgb_pobtasi_stream: the sweep's own
// workspace for the matrix's shape, then the ring (R slots of D, Lo and Ar
// blocks) and the device tip.
constexpr int64_t kRingPobtaf = 4;
constexpr int64_t kRingPobtasi = 32;

int64_t ring_slots(int64_t ring, int64_t dflt, bool even) {
    int64_t r = ring > 0 ? ring : dflt;
    if (even) r -= r % 2;
    return r;
}

struct StreamWs {
    size_t sweep = 0, ringD = 0, ringLo = 0, ringAr = 0, tip = 0, total = 0;
    StreamWs(const sgb_bta* m, size_t sweep_bytes, int64_t R) {
        const size_t es = m->dtype == SGB_F64 ? 8 : 4;
        const size_t b = (size_t)m->b, a = (size_t)m->a;
        Carve c;
        sweep = c.take(sweep_bytes);
        ringD = c.take(es * (size_t)R * b * b);
        ringLo = c.take(es * (size_t)R * b * b);
        ringAr = c.take(es * (size_t)R * a * b);
        tip = c.take(es * a * a);
        total = c.off;
    }
};

// The device-side descriptor of the ring: the sweeps address block i in
// slot (i - off) mod R through Blocks.
sgb_bta ring_desc(const sgb_bta* host, char* ws, const StreamWs& L) {
    sgb_bta d = *host;
    d.diag = ws + L.ringD;
    d.lower = ws + L.ringLo;
    d.arrow = ws + L.ringAr;
    d.tip = ws + L.tip;
    return d;
}

int stream_sizes(const sgb_bta* host, int precision, int64_t ring, bool inverse, int64_t* R, size_t* sweep,
                 size_t* total) {
    int rc = check_bta(host);
    if (rc) return rc;
    const int S = parse_precision(precision, host->dtype);
    if (S < 0) return -S;
    const int Si = parse_inv_slices(precision, S);
    *R = inverse ? ring_slots(ring, kRingPobtasi, true) : ring_slots(ring, kRingPobtaf, false);
    if (*R < 2 || *R > ((int64_t)1 << 20)) return SGB_ERR_SHAPE;
    if (inverse)
        *sweep = host->dtype == SGB_F64 ? PobtasiWs<double>(host, S, Si, *R / 2).total
                                        : PobtasiWs<float>(host, S, Si, *R / 2).total;
    else
        *sweep = host->dtype == SGB_F64 ? PobtafWs<double>(host, S, Si).total : PobtafWs<float>(host, S, Si).total;
    *total = StreamWs(host, *sweep, *R).total;
    return SGB_OK;
}

}  // namespace
}  // namespace sgb

using namespace sgb;

extern "C" {

int sgb_version(void) { return 100; }

const char* sgb_strerror(int code) {
    switch (code) {
        case SGB_OK: return "ok";
        case SGB_ERR_SHAPE: return "invalid shape";
        case SGB_ERR_DTYPE: return "unsupported dtype";
        case SGB_ERR_NOT_SPD: return "matrix is not positive definite";
        case SGB_ERR_TIMEOUT: return "device wait timed out";
        case SGB_ERR_CUDA: return "CUDA runtime error";
        case SGB_ERR_WORKSPACE: return "workspace missing, too small or misaligned";
        case SGB_ERR_ARG: return "invalid argument";
        case SGB_ERR_UNSUPPORTED: return "not supported by this build";
        default: return "unknown error";
    }
}

int sgb_last_cuda_error(void) { return g_last_cuda_error; }

int sgb_pobtaf_workspace_size(const sgb_bta* m, int precision, size_t* bytes) {
    if (cx_dtype(m)) return cx_pobtaf_workspace_size(m, precision, bytes, false);
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    if (S < 0) return -S;
    if (!bytes) return SGB_ERR_ARG;
    const int Si = parse_inv_slices(precision, S);
    *bytes = m->dtype == SGB_F64 ? PobtafWs<double>(m, S, Si).total : PobtafWs<float>(m, S, Si).total;
    return SGB_OK;
}

int sgb_pobtasi_workspace_size(const sgb_bta* m, int precision, size_t* bytes) {
    if (cx_dtype(m)) return cx_pobtasi_workspace_size(m, precision, bytes, false);
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    if (S < 0) return -S;
    if (!bytes) return SGB_ERR_ARG;
    const int Si = parse_inv_slices(precision, S);
    *bytes = m->dtype == SGB_F64 ? PobtasiWs<double>(m, S, Si).total : PobtasiWs<float>(m, S, Si).total;
    return SGB_OK;
}

int sgb_pobtas_workspace_size(const sgb_bta* m, int64_t nrhs, int precision, size_t* bytes) {
    if (cx_dtype(m)) return cx_pobtas_workspace_size(m, nrhs, precision, bytes, false);
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    if (S < 0) return -S;
    if (!bytes) return SGB_ERR_ARG;
    if (nrhs < 0 || nrhs > (1 << 20)) return SGB_ERR_SHAPE;
    *bytes = m->dtype == SGB_F64 ? PobtasWs<double>(m, nrhs).total : PobtasWs<float>(m, nrhs).total;
    return SGB_OK;
}

int sgb_dgemm_workspace_size(int precision, int64_t M, int64_t N, int64_t K, size_t* bytes) {
    const int S = parse_precision(precision, SGB_F64);
    if (S < 0) return -S;
    if (!bytes) return SGB_ERR_ARG;
    if (M < 0 || N < 0 || K < 0 || M > (1 << 20) || N > (1 << 20) || K > (1 << 20)) return SGB_ERR_SHAPE;
    if (S == 0) {
        *bytes = 256;
        return SGB_OK;
    }
    const int64_t mx = M > N ? M : N;
    *bytes = 256 + tc_bound(S, mx, K < kTcMaxK ? K : kTcMaxK, 1);
    return SGB_OK;
}

int sgb_dgemm(int precision, char transA, char transB, int64_t M, int64_t N, int64_t K, double alpha,
              const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
              void* workspace, size_t workspace_bytes, void* stream) {
    const int S = parse_precision(precision, SGB_F64);
    if (S < 0) return -S;
    if ((transA != 'N' && transA != 'T') || (transB != 'N' && transB != 'T')) return SGB_ERR_ARG;
    if (M < 0 || N < 0 || K < 0 || M > (1 << 20) || N > (1 << 20) || K > (1 << 20)) return SGB_ERR_SHAPE;
    if (M == 0 || N == 0) return SGB_OK;
    if (C == nullptr || (K > 0 && (A == nullptr || B == nullptr))) return SGB_ERR_ARG;
    if (ldc < N || (K > 0 && (lda < (transA == 'N' ? K : M) || ldb < (transB == 'N' ? N : K)))) return SGB_ERR_SHAPE;
    size_t need = 0;
    sgb_dgemm_workspace_size(precision, M, N, K, &need);
    int rc = check_ws(workspace, workspace_bytes, need);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    SGB_TRY(cudaMemsetAsync(workspace, 0, sizeof(int32_t), s));
    Ctx cx;
    cx.slices = S;
    cx.tc = (char*)workspace + 256;
    cx.tc_bytes = workspace_bytes - 256;
    cx.status = (int32_t*)workspace;
    // K beyond the exact-accumulation bound runs as consecutive K chunks
    // accumulated into C (beta = 1 after the first chunk).
    const int64_t kchunk = S ? kTcMaxK : (K > 0 ? K : 1);
    int64_t k0 = 0;
    do {
        const int64_t kc = (K - k0) < kchunk ? (K - k0) : kchunk;
        GemmProb<double> p = prob<double>();
        p.M = (int32_t)M;
        p.N = (int32_t)N;
        if (kc > 0) {
            const double* Ak = transA == 'N' ? A + k0 : A + k0 * lda;
            const double* Bk = transB == 'N' ? B + k0 * ldb : B + k0;
            set_term<double>(p, 0, Ak, lda, transA == 'T', Bk, ldb, transB == 'T', kc);
        }
        p.alpha = alpha;
        p.beta = k0 == 0 ? beta : 1.0;
        p.Cin = C;
        p.ldcin = ldc;
        p.Cout = C;
        p.ldc = ldc;
        SGB_TRY(run_gemm<double>(cx, &p, 1, s));
        k0 += kc;
    } while (k0 < K);
    return SGB_OK;
}

int sgb_pobtaf(const sgb_bta* m, int factorize_last_block, int precision, void* workspace,
               size_t workspace_bytes, int32_t* info, void* stream) {
    if (cx_dtype(m))
        return cx_pobtaf(m, factorize_last_block, precision, workspace, workspace_bytes, info,
                         (cudaStream_t)stream, nullptr);
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    if (S < 0) return -S;
    size_t need = 0;
    sgb_pobtaf_workspace_size(m, precision, &need);
    if ((rc = check_ws(workspace, workspace_bytes, need))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (info) SGB_TRY(cudaMemsetAsync(info, 0, sizeof(int32_t), s));
    SGB_TRY(cudaMemsetAsync(workspace, 0, sizeof(int32_t), s));  // status word
    const int Si = parse_inv_slices(precision, S);
    if (m->dtype == SGB_F64) return pobtaf_run<double>(m, factorize_last_block, S, Si, workspace, info, s);
    return pobtaf_run<float>(m, factorize_last_block, S, Si, workspace, info, s);
}

int sgb_pobtasi(const sgb_bta* m, int invert_last_block, int precision, void* workspace, size_t workspace_bytes,
                void* stream) {
    if (cx_dtype(m))
        return cx_pobtasi(m, invert_last_block, precision, workspace, workspace_bytes, (cudaStream_t)stream,
                          nullptr);
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    if (S < 0) return -S;
    size_t need = 0;
    sgb_pobtasi_workspace_size(m, precision, &need);
    if ((rc = check_ws(workspace, workspace_bytes, need))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    SGB_TRY(cudaMemsetAsync(workspace, 0, sizeof(int32_t), s));  // status word
    const int Si = parse_inv_slices(precision, S);
    if (m->dtype == SGB_F64) return pobtasi_run<double>(m, invert_last_block, S, Si, workspace, s);
    return pobtasi_run<float>(m, invert_last_block, S, Si, workspace, s);
}

int sgb_pobtas(const sgb_bta* m, void* rhs, int64_t nrhs, int64_t ldb, char trans, int partial, int precision,
               void* workspace, size_t workspace_bytes, void* stream) {
    if (cx_dtype(m))
        return cx_pobtas(m, rhs, nrhs, ldb, trans, partial, precision, workspace, workspace_bytes,
                         (cudaStream_t)stream, nullptr);
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    if (S < 0) return -S;
    if (trans != 'N' && trans != 'T' && trans != 'C') return SGB_ERR_ARG;
    if (nrhs < 0 || nrhs > (1 << 20) || ldb < nrhs) return SGB_ERR_SHAPE;
    if (nrhs > 0 && rhs == nullptr) return SGB_ERR_ARG;
    size_t need = 0;
    sgb_pobtas_workspace_size(m, nrhs, precision, &need);
    if ((rc = check_ws(workspace, workspace_bytes, need))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (m->dtype == SGB_F64)
        return pobtas_native<double>(m, (double*)rhs, nrhs, ldb, trans, partial, workspace, s);
    return pobtas_native<float>(m, (float*)rhs, nrhs, ldb, trans, partial, workspace, s);
}

int sgb_pobtaf_permuted(const sgb_bta* m, void* buffer, int precision, void* workspace, size_t workspace_bytes,
                        int32_t* info, void* stream) {
    if (cx_dtype(m)) {
        if (buffer == nullptr) return SGB_ERR_ARG;
        if (m->n < 2) return SGB_ERR_SHAPE;
        return cx_pobtaf(m, 1, precision, workspace, workspace_bytes, info, (cudaStream_t)stream, buffer);
    }
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    if (S < 0) return -S;
    const int Si = parse_inv_slices(precision, S);
    if (m->n < 2) return SGB_ERR_SHAPE;
    if (buffer == nullptr) return SGB_ERR_ARG;
    size_t need = 0;
    sgb_pobtaf_permuted_workspace_size(m, precision, &need);
    if ((rc = check_ws(workspace, workspace_bytes, need))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (info) SGB_TRY(cudaMemsetAsync(info, 0, sizeof(int32_t), s));
    SGB_TRY(cudaMemsetAsync(workspace, 0, sizeof(int32_t), s));  // status word
    if (m->dtype == SGB_F64) return pobtaf_permuted_run<double>(m, (double*)buffer, S, Si, workspace, info, s);
    return pobtaf_permuted_run<float>(m, (float*)buffer, S, Si, workspace, info, s);
}

int sgb_pobtaf_permuted_workspace_size(const sgb_bta* m, int precision, size_t* bytes) {
    if (cx_dtype(m)) return cx_pobtaf_workspace_size(m, precision, bytes, true);
    return sgb_pobtaf_workspace_size(m, precision, bytes);
}

int sgb_pobtas_permuted_workspace_size(const sgb_bta* m, int64_t nrhs, int precision, size_t* bytes) {
    if (cx_dtype(m)) return cx_pobtas_workspace_size(m, nrhs, precision, bytes, true);
    return sgb_pobtas_workspace_size(m, nrhs, precision, bytes);
}

int sgb_pobtasi_permuted_workspace_size(const sgb_bta* m, int precision, size_t* bytes) {
    if (cx_dtype(m)) return cx_pobtasi_workspace_size(m, precision, bytes, true);
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    if (S < 0) return -S;
    const int Si = parse_inv_slices(precision, S);
    if (!bytes) return SGB_ERR_ARG;
    *bytes = m->dtype == SGB_F64 ? PobtasiPermWs<double>(m, S, Si).total : PobtasiPermWs<float>(m, S, Si).total;
    return SGB_OK;
}

int sgb_pobtasi_permuted(const sgb_bta* m, void* buffer, int precision, void* workspace, size_t workspace_bytes,
                         void* stream) {
    if (cx_dtype(m)) {
        if (buffer == nullptr) return SGB_ERR_ARG;
        if (m->n < 2) return SGB_ERR_SHAPE;
        return cx_pobtasi(m, 1, precision, workspace, workspace_bytes, (cudaStream_t)stream, buffer);
    }
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    if (S < 0) return -S;
    const int Si = parse_inv_slices(precision, S);
    if (m->n < 2) return SGB_ERR_SHAPE;
    if (buffer == nullptr) return SGB_ERR_ARG;
    size_t need = 0;
    sgb_pobtasi_permuted_workspace_size(m, precision, &need);
    if ((rc = check_ws(workspace, workspace_bytes, need))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    SGB_TRY(cudaMemsetAsync(workspace, 0, sizeof(int32_t), s));  // status word
    if (m->dtype == SGB_F64) return pobtasi_permuted_run<double>(m, (double*)buffer, S, Si, workspace, s);
    return pobtasi_permuted_run<float>(m, (float*)buffer, S, Si, workspace, s);
}

int sgb_pobtas_permuted(const sgb_bta* m, void* buffer, void* rhs, int64_t nrhs, int64_t ldb, char trans,
                        int precision, void* workspace, size_t workspace_bytes, void* stream) {
    if (cx_dtype(m)) {
        if (buffer == nullptr) return SGB_ERR_ARG;
        return cx_pobtas(m, rhs, nrhs, ldb, trans, 0, precision, workspace, workspace_bytes,
                         (cudaStream_t)stream, buffer);
    }
    int rc = check_bta(m);
    if (rc) return rc;
    const int S = parse_precision(precision, m->dtype);
    if (S < 0) return -S;  // the solve runs in the storage precision in either mode
    if (trans != 'N' && trans != 'T' && trans != 'C') return SGB_ERR_ARG;
    if (nrhs < 0 || nrhs > (1 << 20) || ldb < nrhs) return SGB_ERR_SHAPE;
    if ((nrhs > 0 && rhs == nullptr) || buffer == nullptr) return SGB_ERR_ARG;
    size_t need = 0;
    sgb_pobtas_permuted_workspace_size(m, nrhs, precision, &need);
    if ((rc = check_ws(workspace, workspace_bytes, need))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (m->dtype == SGB_F64)
        return pobtas_permuted_run<double>(m, (double*)buffer, (double*)rhs, nrhs, ldb, trans, workspace, s);
    return pobtas_permuted_run<float>(m, (float*)buffer, (float*)rhs, nrhs, ldb, trans, workspace, s);
}

int sgb_bta_symv(const sgb_bta* A, const void* x, int64_t ldx, void* y, int64_t ldy, int64_t nrhs, double alpha,
                 double beta, void* stream) {
    int rc = check_bta(A);
    if (rc) return rc;
    if (nrhs < 0 || nrhs > (1 << 20) || ldx < nrhs || ldy < nrhs) return SGB_ERR_SHAPE;
    if (nrhs == 0) return SGB_OK;
    if (x == nullptr || y == nullptr) return SGB_ERR_ARG;
    const int64_t N = A->n * A->b + A->a;
    const size_t es = A->dtype == SGB_F64 ? 8 : 4;
    const uintptr_t xl = (uintptr_t)x, xh = xl + es * (size_t)((N - 1) * ldx + nrhs);
    const uintptr_t yl = (uintptr_t)y, yh = yl + es * (size_t)((N - 1) * ldy + nrhs);
    if (xl < yh && yl < xh) return SGB_ERR_ARG;  // x and y overlap
    cudaStream_t s = (cudaStream_t)stream;
    if (A->dtype == SGB_F64)
        SGB_TRY(bta_symv<double>(A, (const double*)x, ldx, (double*)y, ldy, nrhs, alpha, beta, s));
    else
        SGB_TRY(bta_symv<float>(A, (const float*)x, ldx, (float*)y, ldy, nrhs, (float)alpha, (float)beta, s));
    return SGB_OK;
}

int sgb_pobtas_refine_workspace_size(const sgb_bta* L, int64_t nrhs, size_t* bytes) {
    int rc = check_bta(L);
    if (rc) return rc;
    if (!bytes) return SGB_ERR_ARG;
    if (nrhs < 0 || nrhs > (1 << 20)) return SGB_ERR_SHAPE;
    *bytes = L->dtype == SGB_F64 ? RefineWs<double>(L, nrhs).total : RefineWs<float>(L, nrhs).total;
    return SGB_OK;
}

int sgb_pobtas_refine(const sgb_bta* A, const sgb_bta* L, void* rhs, int64_t nrhs, int64_t ldb, int iters,
                      void* workspace, size_t workspace_bytes, void* stream) {
    int rc = check_bta(A);
    if (rc) return rc;
    if ((rc = check_bta(L))) return rc;
    if (A->dtype != L->dtype || A->n != L->n || A->b != L->b || A->a != L->a) return SGB_ERR_SHAPE;
    if (nrhs < 0 || nrhs > (1 << 20) || ldb < nrhs) return SGB_ERR_SHAPE;
    if (iters < 0 || iters > 100) return SGB_ERR_ARG;
    if (nrhs > 0 && rhs == nullptr) return SGB_ERR_ARG;
    size_t need = 0;
    sgb_pobtas_refine_workspace_size(L, nrhs, &need);
    if ((rc = check_ws(workspace, workspace_bytes, need))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (A->dtype == SGB_F64) return pobtas_refine_run<double>(A, L, (double*)rhs, nrhs, ldb, iters, workspace, s);
    return pobtas_refine_run<float>(A, L, (float*)rhs, nrhs, ldb, iters, workspace, s);
}

// Host-resident stacks: `host` holds the caller's (pinned) host arrays, `dev`
// a device copy of the same shape that the sweep works in.
int check_host_pair(const sgb_bta* host, const sgb_bta* dev) {
    int rc = check_bta(host);
    if (rc) return rc;
    if ((rc = check_bta(dev))) return rc;
    if (host->dtype != dev->dtype || host->n != dev->n || host->b != dev->b || host->a != dev->a)
        return SGB_ERR_SHAPE;
    return SGB_OK;
}

int sgb_pobtaf_host(const sgb_bta* host, const sgb_bta* dev, int factorize_last_block, int precision,
                    void* workspace, size_t workspace_bytes, int32_t* info, void* stream) {
    int rc = check_host_pair(host, dev);
    if (rc) return rc;
    const int S = parse_precision(precision, dev->dtype);
    if (S < 0) return -S;
    size_t need = 0;
    sgb_pobtaf_workspace_size(dev, precision, &need);
    if ((rc = check_ws(workspace, workspace_bytes, need))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (info) SGB_TRY(cudaMemsetAsync(info, 0, sizeof(int32_t), s));
    SGB_TRY(cudaMemsetAsync(workspace, 0, sizeof(int32_t), s));  // status word
    HostLink hl;
    hl.h = host;
    hl.d = dev;
    hl.ascending = true;
    hl.es = dev->dtype == SGB_F64 ? 8 : 4;
    const int Si = parse_inv_slices(precision, S);
    if (dev->dtype == SGB_F64)
        return pobtaf_run<double>(dev, factorize_last_block, S, Si, workspace, info, s, &hl);
    return pobtaf_run<float>(dev, factorize_last_block, S, Si, workspace, info, s, &hl);
}

int sgb_pobtaf_stream_workspace_size(const sgb_bta* host, int precision, int64_t ring, size_t* bytes) {
    if (cx_dtype(host)) return SGB_ERR_UNSUPPORTED;
    if (!bytes) return SGB_ERR_ARG;
    int64_t R = 0;
    size_t sweep = 0;
    return stream_sizes(host, precision, ring, false, &R, &sweep, bytes);
}

int sgb_pobtasi_stream_workspace_size(const sgb_bta* host, int precision, int64_t ring, size_t* bytes) {
    if (cx_dtype(host)) return SGB_ERR_UNSUPPORTED;
    if (!bytes) return SGB_ERR_ARG;
    int64_t R = 0;
    size_t sweep = 0;
    return stream_sizes(host, precision, ring, true, &R, &sweep, bytes);
}

int sgb_pobtaf_stream(const sgb_bta* host, int factorize_last_block, int precision, int64_t ring, void* workspace,
                      size_t workspace_bytes, int32_t* info, void* stream) {
    if (cx_dtype(host)) return SGB_ERR_UNSUPPORTED;
    int64_t R = 0;
    size_t sweep = 0, total = 0;
    int rc = stream_sizes(host, precision, ring, false, &R, &sweep, &total);
    if (rc) return rc;
    if ((rc = check_ws(workspace, workspace_bytes, total))) return rc;
    const int S = parse_precision(precision, host->dtype);
    const int Si = parse_inv_slices(precision, S);
    const StreamWs L(host, sweep, R);
    const sgb_bta dm = ring_desc(host, (char*)workspace, L);
    cudaStream_t s = (cudaStream_t)stream;
    if (info) SGB_TRY(cudaMemsetAsync(info, 0, sizeof(int32_t), s));
    SGB_TRY(cudaMemsetAsync(workspace, 0, sizeof(int32_t), s));  // status word
    HostRing hr;
    hr.h = host;
    hr.dD = (char*)dm.diag;
    hr.dLo = (char*)dm.lower;
    hr.dAr = (char*)dm.arrow;
    hr.dT = (char*)dm.tip;
    hr.R = R;
    hr.off = 0;
    hr.ascending = true;
    hr.es = host->dtype == SGB_F64 ? 8 : 4;
    if (host->dtype == SGB_F64)
        return pobtaf_run<double>(&dm, factorize_last_block, S, Si, workspace, info, s, &hr, nullptr, nullptr, R);
    return pobtaf_run<float>(&dm, factorize_last_block, S, Si, workspace, info, s, &hr, nullptr, nullptr, R);
}

int sgb_pobtasi_stream(const sgb_bta* host, int invert_last_block, int precision, int64_t ring, void* workspace,
                       size_t workspace_bytes, void* stream) {
    if (cx_dtype(host)) return SGB_ERR_UNSUPPORTED;
    int64_t R = 0;
    size_t sweep = 0, total = 0;
    int rc = stream_sizes(host, precision, ring, true, &R, &sweep, &total);
    if (rc) return rc;
    if ((rc = check_ws(workspace, workspace_bytes, total))) return rc;
    const int S = parse_precision(precision, host->dtype);
    const int Si = parse_inv_slices(precision, S);
    const StreamWs L(host, sweep, R);
    const sgb_bta dm = ring_desc(host, (char*)workspace, L);
    cudaStream_t s = (cudaStream_t)stream;
    SGB_TRY(cudaMemsetAsync(workspace, 0, sizeof(int32_t), s));  // status word
    HostRing hr;
    hr.h = host;
    hr.dD = (char*)dm.diag;
    hr.dLo = (char*)dm.lower;
    hr.dAr = (char*)dm.arrow;
    hr.dT = (char*)dm.tip;
    hr.R = R;
    hr.off = invert_last_block ? host->n : host->n - 1;  // the sweep's chunk alignment
    hr.ascending = false;
    hr.es = host->dtype == SGB_F64 ? 8 : 4;
    if (host->dtype == SGB_F64)
        return pobtasi_run<double>(&dm, invert_last_block, S, Si, workspace, s, &hr, nullptr, R);
    return pobtasi_run<float>(&dm, invert_last_block, S, Si, workspace, s, &hr, nullptr, R);
}

int sgb_pobtasi_host(const sgb_bta* host, const sgb_bta* dev, int invert_last_block, int precision,
                     void* workspace, size_t workspace_bytes, void* stream) {
    int rc = check_host_pair(host, dev);
    if (rc) return rc;
    const int S = parse_precision(precision, dev->dtype);
    if (S < 0) return -S;
    size_t need = 0;
    sgb_pobtasi_workspace_size(dev, precision, &need);
    if ((rc = check_ws(workspace, workspace_bytes, need))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    SGB_TRY(cudaMemsetAsync(workspace, 0, sizeof(int32_t), s));  // status word
    HostLink hl;
    hl.h = host;
    hl.d = dev;
    hl.ascending = false;
    hl.es = dev->dtype == SGB_F64 ? 8 : 4;
    const int Si = parse_inv_slices(precision, S);
    if (dev->dtype == SGB_F64) return pobtasi_run<double>(dev, invert_last_block, S, Si, workspace, s, &hl);
    return pobtasi_run<float>(dev, invert_last_block, S, Si, workspace, s, &hl);
}

}  // extern "C"
