// Batched execution of many independent BTA matrices of uneven shapes.
//
// A plan distributes the matrices over worker streams (longest-processing-
// time first on a cost estimate), captures the per-matrix sweeps
//   pobtaf -> [pobtas N, pobtas T] -> [pobtasi]
// of every matrix into one CUDA graph (fork/join through events), and
// replays that graph on the caller's stream with one cudaGraphLaunch.
// Matrices on the same worker stream run one after another and share that
// stream's slice of the workspace; different streams run concurrently and
// fill the GPU with independent block chains.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <string.h>
#include <vector>

#include "sgb_internal.cuh"

// CTAs of a captured column-block launch unless the plan asks otherwise.
constexpr int kPlanPanelGrid = 24;

struct sgb_batch_plan {
    int count = 0;
    int nstreams = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int32_t* info = nullptr;  // device, count entries (in the workspace)
};

namespace {

struct Item {
    sgb_bta m;
    void* rhs;
    int64_t nrhs;
    int precision;
    double cost;
    size_t ws;
};

size_t item_ws(const Item& it, int ops) {
    // sized as the plan's capture runs the item (a panel grid set)
    sgb::set_capture_panel_grid(kPlanPanelGrid);
    const size_t need = sgb::plan_item_ws(&it.m, ops, it.precision, it.nrhs);
    sgb::set_capture_panel_grid(0);
    return (need + 255) / 256 * 256;
}

// Rough device time: FP64 work at ~0.6 TF/s, FP32 at ~8x that, plus a fixed
// latency per 32-wide diagonal tile (the sequential pivot chain).
double item_cost(const sgb_bta& m) {
    // complex matrices run as their real embedding (blocks 2b, arrow 2a)
    const bool cx = m.dtype == SGB_C64 || m.dtype == SGB_C128;
    const double n = (double)m.n, b = (cx ? 2.0 : 1.0) * m.b, a = (cx ? 2.0 : 1.0) * m.a;
    const double fl = n * (26.0 / 3.0 * b * b * b + 10.0 * a * b * b + 3.0 * a * a * b);
    const double rate = (m.dtype == SGB_F64 || m.dtype == SGB_C128) ? 0.6e12 : 4.8e12;
    const double tiles = n * std::ceil(b / 32.0);
    return fl / rate + tiles * 30e-6;
}

int validate(const sgb_bta* mats, void* const* rhs, const int64_t* nrhs, int count, int ops,
             const int* precisions, std::vector<Item>& items) {
    if (count < 0 || (count > 0 && mats == nullptr)) return SGB_ERR_ARG;
    if ((ops & ~(SGB_OP_POBTAF | SGB_OP_POBTASI | SGB_OP_POBTAS)) != 0 || ops == 0) return SGB_ERR_ARG;
    items.resize(count);
    for (int i = 0; i < count; ++i) {
        Item& it = items[i];
        it.m = mats[i];
        it.rhs = rhs ? rhs[i] : nullptr;
        it.nrhs = nrhs ? nrhs[i] : 0;
        it.precision = precisions ? precisions[i] : SGB_PREC_NATIVE;
        if ((ops & SGB_OP_POBTAS) && it.nrhs > 0 && it.rhs == nullptr) return SGB_ERR_ARG;
        if (it.nrhs < 0) return SGB_ERR_SHAPE;
        size_t x = 0;
        int rc = sgb_pobtaf_workspace_size(&it.m, it.precision, &x);
        if (rc) return rc;
        it.cost = item_cost(it.m);
        it.ws = item_ws(it, ops);
    }
    return SGB_OK;
}

// LPT assignment: biggest first onto the least loaded stream.
std::vector<int> assign(const std::vector<Item>& items, int nstreams) {
    std::vector<int> order(items.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return items[x].cost > items[y].cost; });
    std::vector<double> load(nstreams, 0.0);
    std::vector<int> where(items.size(), 0);
    for (int i : order) {
        const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        where[i] = k;
        load[k] += items[i].cost;
    }
    return where;
}

struct Layout {
    std::vector<size_t> stream_off, stream_bytes;
    size_t info_off = 0, total = 0;
};

Layout layout(const std::vector<Item>& items, const std::vector<int>& where, int nstreams) {
    Layout L;
    L.stream_off.assign(nstreams, 0);
    L.stream_bytes.assign(nstreams, 0);
    for (size_t i = 0; i < items.size(); ++i)
        L.stream_bytes[where[i]] = std::max(L.stream_bytes[where[i]], items[i].ws);
    size_t off = 0;
    L.info_off = off;
    off += (items.size() * sizeof(int32_t) + 255) / 256 * 256;
    for (int k = 0; k < nstreams; ++k) {
        L.stream_off[k] = off;
        off += L.stream_bytes[k];
    }
    L.total = off < 256 ? 256 : off;
    return L;
}

}  // namespace

extern "C" {

int sgb_batch_workspace_size(const sgb_bta* mats, void* const* rhs, const int64_t* nrhs, int count, int ops,
                             const int* precisions, int nstreams, size_t* bytes) {
    if (!bytes || nstreams < 1 || nstreams > 256) return SGB_ERR_ARG;
    std::vector<Item> items;
    int rc = validate(mats, rhs, nrhs, count, ops, precisions, items);
    if (rc) return rc;
    const int ns = std::max(1, std::min(nstreams, count));
    *bytes = layout(items, assign(items, ns), ns).total;
    return SGB_OK;
}

int sgb_batch_plan_create(const sgb_bta* mats, void* const* rhs, const int64_t* nrhs, int count, int ops,
                          const int* precisions, int nstreams, void* workspace, size_t workspace_bytes,
                          sgb_batch_plan** out) {
    return sgb_batch_plan_create_ex(mats, rhs, nrhs, count, ops, precisions, nstreams, 0, 0, workspace,
                                    workspace_bytes, out);
}

int sgb_batch_plan_create_ex(const sgb_bta* mats, void* const* rhs, const int64_t* nrhs, int count, int ops,
                             const int* precisions, int nstreams, int panel_ctas, int options, void* workspace,
                             size_t workspace_bytes, sgb_batch_plan** out) {
    if (!out || nstreams < 1 || nstreams > 256) return SGB_ERR_ARG;
    if (panel_ctas < 0 || panel_ctas > 1024) return SGB_ERR_ARG;
    if ((options & ~SGB_BATCH_TC_KSPLIT) != 0) return SGB_ERR_ARG;
    const int pgrid = panel_ctas == 0 ? kPlanPanelGrid : panel_ctas;
    *out = nullptr;
    std::vector<Item> items;
    int rc = validate(mats, rhs, nrhs, count, ops, precisions, items);
    if (rc) return rc;
    const int ns = std::max(1, std::min(nstreams, count));
    const std::vector<int> where = assign(items, ns);
    const Layout L = layout(items, where, ns);
    if (workspace == nullptr || workspace_bytes < L.total || ((uintptr_t)workspace) % 256) return SGB_ERR_WORKSPACE;

    sgb::tc_prepare();  // kernel attributes are set before capture
    sgb_batch_plan* plan = new sgb_batch_plan();
    plan->count = count;
    plan->nstreams = ns;
    plan->info = (int32_t*)((char*)workspace + L.info_off);

    std::vector<cudaStream_t> streams(ns + 1, nullptr);
    std::vector<cudaEvent_t> events(ns + 1, nullptr);
    cudaError_t e = cudaSuccess;
    for (int k = 0; k <= ns && e == cudaSuccess; ++k) {
        e = cudaStreamCreateWithFlags(&streams[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&events[k], cudaEventDisableTiming);
    }
    cudaStream_t origin = streams[ns];
    bool capturing = false;
    if (e == cudaSuccess) {
        e = cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal);
        capturing = e == cudaSuccess;
    }
    // pobtaf blocks of b > 64 become one cooperative column-block launch of
    // pgrid CTAs each (a few run side by side; a grid too small for the
    // kernel's roles falls back to the launch-based tile sweep); smaller
    // blocks keep the tile sweep
    sgb::set_capture_panel_grid(pgrid);
    sgb::set_capture_tc_split((options & SGB_BATCH_TC_KSPLIT) != 0);
    if (e == cudaSuccess) e = cudaEventRecord(events[ns], origin);
    for (int k = 0; k < ns && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(streams[k], events[ns], 0);
    // enqueue every matrix on its stream, biggest first within a stream
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return items[x].cost > items[y].cost; });
    for (int idx = 0; idx < count && e == cudaSuccess && rc == SGB_OK; ++idx) {
        const int i = order[idx];
        const Item& it = items[i];
        const int k = where[i];
        void* ws = (char*)workspace + L.stream_off[k];
        const size_t wsb = L.stream_bytes[k];
        void* s = (void*)streams[k];
        rc = sgb::plan_item(&it.m, ops, it.precision, it.rhs, it.nrhs, ws, wsb, plan->info + i, (cudaStream_t)s);
    }
    for (int k = 0; k < ns && e == cudaSuccess && rc == SGB_OK; ++k) {
        e = cudaEventRecord(events[k], streams[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(origin, events[k], 0);
    }
    sgb::set_capture_panel_grid(0);
    sgb::set_capture_tc_split(false);
    if (capturing) {
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(origin, &g);
        if (e == cudaSuccess) e = e2;
        plan->graph = g;
    }
    if (e == cudaSuccess && rc == SGB_OK) e = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
    for (int k = 0; k <= ns; ++k) {
        if (events[k]) cudaEventDestroy(events[k]);
        if (streams[k]) cudaStreamDestroy(streams[k]);
    }
    if (rc == SGB_OK && e != cudaSuccess) rc = SGB_ERR_CUDA;
    if (rc != SGB_OK) {
        sgb_batch_plan_destroy(plan);
        return rc;
    }
    *out = plan;
    return SGB_OK;
}

int sgb_batch_run(sgb_batch_plan* plan, void* stream) {
    if (!plan || !plan->exec) return SGB_ERR_ARG;
    if (cudaGraphLaunch(plan->exec, (cudaStream_t)stream) != cudaSuccess) return SGB_ERR_CUDA;
    return SGB_OK;
}

const int32_t* sgb_batch_info(const sgb_batch_plan* plan) { return plan ? plan->info : nullptr; }

int sgb_batch_plan_destroy(sgb_batch_plan* plan) {
    if (!plan) return SGB_OK;
    if (plan->exec) cudaGraphExecDestroy(plan->exec);
    if (plan->graph) cudaGraphDestroy(plan->graph);
    delete plan;
    return SGB_OK;
}

}  // extern "C"
