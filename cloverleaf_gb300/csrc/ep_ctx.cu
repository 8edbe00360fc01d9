// ep_ctx.cu -- host driver behind the C ABI declared in include/ep_gb300.h.
//
// Owns the device copies of the graph CSR, the feature CSR, the feature table
// and Adam moments, plus per-batch scratch, and sequences the per-batch
// kernels (see ep_internal.h) on the context's stream.  In the FUSED form one
// batch is captured once as a CUDA graph and replayed for every batch of every
// pass; the kernels read their batch index, step and learning rate from a
// device-resident BatchState that the last kernel of the batch advances.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ep_gb300.h"
#include "ep_internal.h"

using namespace ep;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBuf() { if (p) cudaFree(p); }
    // Grows to at least n bytes (contents not preserved).  Returns false on OOM.
    bool ensure(size_t n) {
        if (n <= bytes && p) return true;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (cudaMalloc(&p, n ? n : 16) != cudaSuccess) { cudaGetLastError(); return false; }
        bytes = n ? n : 16;
        return true;
    }
    template <typename X> X* as() const { return (X*)p; }
};

uint32_t pick_vpl(uint32_t dims) {
    const uint32_t need = (dims + 31) / 32;
    uint32_t v = 1;
    while (v < need) v <<= 1;
    return v;
}

uint32_t bits_for(uint64_t n) {  // bits needed to represent n-1
    uint32_t b = 0;
    while (n > 1 && ((n - 1) >> b)) ++b;
    return b;
}

}  // namespace

struct ep_ctx {
    ep_config cfg{};
    int device = 0;
    cudaStream_t stream = nullptr;
    // side branch of captured batches: the loss and k_batch_end run beside
    // the sort (see issue_train_batch)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_loss = nullptr, ev_join = nullptr, ev_sorted = nullptr;
    // second branch: a batch's fix-ups beside the next batch's sampling
    cudaStream_t fix = nullptr;
    cudaStream_t fix2 = nullptr;   // the long spans' fix-ups, beside the short ones on `fix`
    cudaEvent_t ev_red = nullptr, ev_fix = nullptr, ev_fix2 = nullptr;
    bool fix_pending = false;   // the last issued fix-ups have not been joined yet
    std::string err;

    // sizes
    uint64_t n_nodes = 0, n_edges = 0, n_fids = 0;
    uint32_t n_feat = 0, max_feat = 0, max_deg = 0;
    uint32_t dims = 0, dpad = 0, vpl = 1, R = 0, NR = 2, Bcap = 0, Kcap = 0;
    int tt = TT_F32;
    bool graph_ok = false, feats_ok = false, table_ok = false, has_w = false;

    // device data
    DevBuf row, cols, wcdf, fptr, fids, table, m, v, train_ids, valid_ids;
    uint32_t n_train = 0, n_valid = 0, steps_per_pass = 0;
    uint64_t total_steps = 0, warmup = 0;

    // per-batch scratch
    DevBuf st, st_eval, st_inj;
    DevBuf anchors, nbr, nbr_w, nbr_cnt, neg, occ, dir, dir16, scale, valid, loss, status, deferred;
    DevBuf item_f, item_src, item_c, key_alt, idx, idx_alt, hist;
    DevBuf carry_head, carry_tail, carry_f, carry_flags, long_list, gdense, touched, n_touched, packed, xfer, bound;
    DevBuf check;   // CSR validation result / bound histogram scratch
    uint32_t long_cap = 0;   // owner chunks per parity in long_list
    uint64_t items_cap = 0;
    uint32_t buf_B = 0, buf_K = 0, buf_es = 0;
    uint32_t chunk = 128;
    // FUSED form's Adam placement: 0 = by the reducing warp as each feature
    // closes; 1 = gradient rows, then a separate Adam kernel; 2 = queued in
    // the reducing warp's shared memory and updated four rows at a time
    int fused_mode = 2;
    // mode 3's warp-specialised reduction: reducing warps, Adam warps and
    // ring slots per CTA
    uint32_t ring_pw = 12, ring_cw = 4, ring_slots = 32;
    // persistent staged gather: CTAs of its grid (0 = one warp per anchor)
    uint32_t gather_ctas = 0;
    // the queue reducer's resident CTAs per SM (4, or 5 with fewer registers)
    uint32_t queue_ctas = 4;
    // persistent reducer grid (CTAs whose warps take chunks from a work
    // counter); 0 = one warp per chunk
    uint32_t red_ctas = 0;
    // warps per CTA of the one-warp-per-anchor gather (1-8): small CTAs free
    // their slots sooner when anchors differ in work (2: forward 0.164 ->
    // 0.150 ms per batch on the 10M-node graph)
    uint32_t gather_warps = 2;
    // warps per CTA of the sampler (1-8)
    uint32_t sample_warps = 8;
    bool tuned = false;         // autotuner has chosen chunk / fused_mode
    bool prepared = false;
    cudaGraphExec_t gexec = nullptr;
    cudaGraphExec_t gexec_run = nullptr;   // graph_batches consecutive batches
    std::map<uint32_t, cudaGraphExec_t> gexec_rem;   // 2 .. graph_batches - 1 consecutive batches (a run's remainder)
    uint32_t graph_batches = 16;
    uint32_t* sorted_keys = nullptr;
    uint2* sorted_vals = nullptr;
    BatchState* h_st = nullptr;   // pinned mirror

    // host-side view of the pass sequence (mirrors the device BatchState)
    uint32_t host_pass = 1, host_batch = 0;
    uint64_t launches = 0;   // kernels issued by training batches (graph replays count their kernels)
    bool state_ok = false;

    // autograd state
    DevBuf ag_table;
    int ag_precision = -1;
    uint32_t ag_n = 0, ag_K = 0;
    const void* ag_table_ptr = nullptr;

    ~ep_ctx() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (gexec_run) cudaGraphExecDestroy(gexec_run);
        for (auto& kv : gexec_rem) cudaGraphExecDestroy(kv.second);
        if (h_st) cudaFreeHost(h_st);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (ev_loss) cudaEventDestroy(ev_loss);
        if (ev_sorted) cudaEventDestroy(ev_sorted);
        if (ev_red) cudaEventDestroy(ev_red);
        if (ev_fix) cudaEventDestroy(ev_fix);
        if (ev_fix2) cudaEventDestroy(ev_fix2);
        if (fix) cudaStreamDestroy(fix);
        if (fix2) cudaStreamDestroy(fix2);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }

    int fail(int code, const char* fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what) {
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? EP_ERR_OOM : EP_ERR_CUDA, "%s: %s", what,
                    cudaGetErrorString(e));
    }
    void drop_graph() {
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        if (gexec_run) { cudaGraphExecDestroy(gexec_run); gexec_run = nullptr; }
        for (auto& kv : gexec_rem) cudaGraphExecDestroy(kv.second);
        gexec_rem.clear();
    }
};

static std::string g_create_err;

#define CK(call, what)                                 \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return c->cuda_fail(e_, what); \
    } while (0)

extern "C" void ep_config_default(ep_config* cfg) {
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->abi_version = EP_ABI_VERSION;
    cfg->alpha = 0.9f;
    cfg->loss = EP_LOSS_MARGIN;
    cfg->gamma = 1.f;
    cfg->negatives = 1;
    cfg->batch_size = 50;
    cfg->dims = 100;
    cfg->passes = 100;
    cfg->seed = 20222022ull;
    cfg->max_nodes_kind = EP_SAMPLE_ALL;
    cfg->max_features_kind = EP_SAMPLE_ALL;
    cfg->loss_weighting = EP_LW_NONE;
    cfg->loss_weighting_exp = 1.f;
    cfg->valid_pct = 0.1f;
    cfg->form = EP_FORM_PLAIN_FP32;
    cfg->grad_mode = EP_GRAD_REFERENCE;
    cfg->use_graphs = 1;
    cfg->autotune = 1;
    cfg->ppr_restart_p = 0.5f;
}

extern "C" int ep_create(const ep_config* cfg, ep_ctx** out) {
    if (!cfg || !out) { g_create_err = "null argument"; return EP_ERR_INVALID_ARG; }
    *out = nullptr;
    if (cfg->abi_version != EP_ABI_VERSION) { g_create_err = "abi_version mismatch"; return EP_ERR_INVALID_ARG; }
    if (cfg->dims == 0 || cfg->dims > 512) { g_create_err = "dims must be in [1, 512]"; return EP_ERR_INVALID_ARG; }
    if (cfg->batch_size == 0) { g_create_err = "batch_size must be > 0"; return EP_ERR_INVALID_ARG; }
    if (cfg->negatives == 0 || cfg->negatives > 1024) { g_create_err = "negatives must be in [1, 1024]"; return EP_ERR_INVALID_ARG; }
    if (cfg->loss < EP_LOSS_MARGIN || cfg->loss > EP_LOSS_PPR) { g_create_err = "unknown loss"; return EP_ERR_INVALID_ARG; }
    if (cfg->loss == EP_LOSS_PPR && !(cfg->ppr_restart_p >= 0.f && cfg->ppr_restart_p <= 1.f)) {
        g_create_err = "PPR restart probability must be in [0, 1]";
        return EP_ERR_INVALID_ARG;
    }
    if (cfg->max_nodes < 0.f || cfg->max_features < 0.f) {
        g_create_err = "max_nodes / max_features must be either None, or (0, N)";
        return EP_ERR_INVALID_ARG;
    }
    if (cfg->max_nodes_kind == EP_SAMPLE_PROB && !(cfg->max_nodes > 0.f && cfg->max_nodes < 1.f)) {
        g_create_err = "probability max_nodes must be in (0, 1)";
        return EP_ERR_INVALID_ARG;
    }
    if (cfg->valid_pct < 0.f || cfg->valid_pct >= 1.f) { g_create_err = "valid_pct must be in [0, 1)"; return EP_ERR_INVALID_ARG; }
    if (cfg->max_features_kind == EP_SAMPLE_PROB && !(cfg->max_features > 0.f && cfg->max_features < 1.f)) {
        g_create_err = "probability max_features must be in (0, 1)";
        return EP_ERR_INVALID_ARG;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        g_create_err = "no CUDA device";
        return EP_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= ndev) { g_create_err = "device ordinal out of range"; return EP_ERR_INVALID_ARG; }
    ep_ctx* c = new ep_ctx();
    c->cfg = *cfg;
    c->device = cfg->device;
    // the main stream (gathers, loss, reduction: the critical path) at the
    // highest priority, the side branch (items, sort, batch end) at the lowest
    int prio_lo = 0, prio_hi = 0;
    if (cudaSetDevice(c->device) != cudaSuccess || cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c->fix, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c->fix2, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_red, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fix, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fix2, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_loss, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_sorted, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost((void**)&c->h_st, sizeof(BatchState)) != cudaSuccess || reduce_kernels_setup() != cudaSuccess) {
        g_create_err = std::string("CUDA setup failed: ") + cudaGetErrorString(cudaGetLastError());
        delete c;
        return EP_ERR_CUDA;
    }
    c->dims = cfg->dims;
    c->vpl = pick_vpl(cfg->dims);
    c->dpad = ((cfg->dims + c->vpl - 1) / c->vpl) * c->vpl;
    c->tt = cfg->form == EP_FORM_FUSED_BF16 ? TT_BF16 : TT_F32;
    c->R = cfg->negatives;
    c->NR = c->R + 2;
    if (const char* gb = getenv("EP_GRAPH_BATCHES")) {   // batches per replayed graph (tuning)
        const long v = atol(gb);
        if (v >= 1 && v <= 1024) c->graph_batches = (uint32_t)v;
    }
    if (const char* fm = getenv("EP_FUSED_MODE")) {   // (tuning)
        const int v = atoi(fm);
        if (v >= 0 && v <= 3) c->fused_mode = v;
    }
    if (const char* e = getenv("EP_RING_PW")) { const long v = atol(e); if (v >= 1 && v <= 15) c->ring_pw = (uint32_t)v; }
    if (const char* e = getenv("EP_RING_CW")) { const long v = atol(e); if (v >= 1 && v <= 15) c->ring_cw = (uint32_t)v; }
    if (const char* e = getenv("EP_RING_SLOTS")) { const long v = atol(e); if (v >= 2 && v <= 64) c->ring_slots = (uint32_t)v; }
    if (const char* e = getenv("EP_GATHER_CTAS")) { const long v = atol(e); if (v >= 0 && v <= 65536) c->gather_ctas = (uint32_t)v; }
    if (const char* e = getenv("EP_QUEUE_CTAS")) { const long v = atol(e); if (v == 4 || v == 5) c->queue_ctas = (uint32_t)v; }
    if (const char* e = getenv("EP_RED_CTAS")) { const long v = atol(e); if (v >= 0 && v <= 65536) c->red_ctas = (uint32_t)v; }
    if (const char* e = getenv("EP_GATHER_WARPS")) { const long v = atol(e); if (v >= 1 && v <= 8) c->gather_warps = (uint32_t)v; }
    if (const char* e = getenv("EP_SAMPLE_WARPS")) { const long v = atol(e); if (v >= 1 && v <= 8) c->sample_warps = (uint32_t)v; }
    // a launch shape set by hand is used as given: no tuning
    for (const char* k : {"EP_FUSED_MODE", "EP_REDUCE_CHUNK", "EP_GATHER_CTAS", "EP_QUEUE_CTAS", "EP_RED_CTAS", "EP_GATHER_WARPS", "EP_RING_PW",
                          "EP_RING_CW", "EP_RING_SLOTS"})
        if (getenv(k)) c->cfg.autotune = 0;
    if (const char* ch = getenv("EP_REDUCE_CHUNK")) {   // reducer items per warp (tuning)
        const long v = atol(ch);
        if (v >= 32 && v <= (1l << 20)) c->chunk = (uint32_t)v;
    }
    *out = c;
    return EP_OK;
}

extern "C" const char* ep_last_error(const ep_ctx* c) { return c ? c->err.c_str() : g_create_err.c_str(); }

extern "C" void ep_destroy(ep_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    delete c;
}

// CSR validation on the device, after the upload: row pointers must not
// decrease and every id must be below id_bound.  The first offending row and
// id position (or ~0) and the longest row come back in one small copy.
struct CsrCheck {
    unsigned long long bad_row, bad_id, max_row;
};

__global__ void k_check_csr(uint64_t n, const uint64_t* __restrict__ ptr, const uint32_t* __restrict__ ids,
                            uint64_t m, uint64_t id_bound, CsrCheck* out) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long mx = 0;
    for (uint64_t i = tid; i < n; i += stride) {
        const uint64_t a = ptr[i], b = ptr[i + 1];
        if (b < a) atomicMin(&out->bad_row, (unsigned long long)i);
        else mx = b - a > mx ? b - a : mx;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = y > mx ? y : mx;
    }
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(&out->max_row, mx);
    for (uint64_t j = tid; j < m; j += stride)
        if (ids[j] >= id_bound) atomicMin(&out->bad_id, (unsigned long long)j);
}

// Runs k_check_csr over uploaded arrays; fails with the first offence.
static int check_csr(ep_ctx* c, uint64_t n, const uint64_t* d_ptr, const uint32_t* d_ids, uint64_t m,
                     uint64_t id_bound, const char* what, uint32_t* max_row) {
    if (!c->check.ensure(65536 * 12)) return c->fail(EP_ERR_OOM, "scratch allocation failed");
    CsrCheck* dc = c->check.as<CsrCheck>();
    const CsrCheck init{~0ull, ~0ull, 0ull};
    CK(cudaMemcpyAsync(dc, &init, sizeof(init), cudaMemcpyHostToDevice, c->stream), "validate");
    k_check_csr<<<152 * 8, 256, 0, c->stream>>>(n, d_ptr, d_ids, m, id_bound, dc);
    CK(cudaGetLastError(), "validate");
    CsrCheck r;
    CK(cudaMemcpyAsync(&r, dc, sizeof(r), cudaMemcpyDeviceToHost, c->stream), "validate");
    CK(cudaStreamSynchronize(c->stream), "validate");
    if (r.bad_row != ~0ull)
        return c->fail(EP_ERR_INVALID_ARG, "%s: row pointers decrease at row %llu", what, r.bad_row);
    if (r.bad_id != ~0ull) return c->fail(EP_ERR_INVALID_ARG, "%s: id at %llu out of range", what, r.bad_id);
    if (r.max_row > 0xffffffffull) return c->fail(EP_ERR_INVALID_ARG, "%s: row too long", what);
    *max_row = (uint32_t)r.max_row;
    return EP_OK;
}

extern "C" int ep_upload_graph(ep_ctx* c, uint64_t n_nodes, const uint64_t* row_ptr, const uint32_t* cols,
                               const float* w_cdf) {
    if (!c) return EP_ERR_INVALID_ARG;
    if (!row_ptr || (!cols && n_nodes && row_ptr[n_nodes])) return c->fail(EP_ERR_INVALID_ARG, "null graph arrays");
    if (n_nodes == 0 || n_nodes > 0xfffffffeull) return c->fail(EP_ERR_INVALID_ARG, "n_nodes must be in [1, 2^32-1)");
    if (c->feats_ok && n_nodes != c->n_nodes) return c->fail(EP_ERR_INVALID_ARG, "graph and features disagree on node count");
    if (row_ptr[0] != 0) return c->fail(EP_ERR_INVALID_ARG, "graph: row pointer must start at 0");
    cudaSetDevice(c->device);
    const uint64_t E = row_ptr[n_nodes];
    c->graph_ok = false;     // the device copy is replaced below; valid again once checked
    c->prepared = false;
    c->drop_graph();
    if (!c->row.ensure((n_nodes + 1) * 8) || !c->cols.ensure(E * 4) || !c->wcdf.ensure(E * 4))
        return c->fail(EP_ERR_OOM, "graph allocation failed");
    CK(cudaMemcpyAsync(c->row.p, row_ptr, (n_nodes + 1) * 8, cudaMemcpyHostToDevice, c->stream), "upload row_ptr");
    if (E) CK(cudaMemcpyAsync(c->cols.p, cols, E * 4, cudaMemcpyHostToDevice, c->stream), "upload cols");
    if (E && w_cdf) CK(cudaMemcpyAsync(c->wcdf.p, w_cdf, E * 4, cudaMemcpyHostToDevice, c->stream), "upload weights");
    c->has_w = w_cdf != nullptr;
    uint32_t mx = 0;
    int rc = check_csr(c, n_nodes, c->row.as<uint64_t>(), c->cols.as<uint32_t>(), E, n_nodes, "graph", &mx);
    if (rc) return rc;
    c->n_nodes = n_nodes;
    c->n_edges = E;
    c->max_deg = mx;
    c->graph_ok = true;
    c->prepared = false;
    c->drop_graph();
    return EP_OK;
}

extern "C" int ep_upload_features(ep_ctx* c, uint64_t n_nodes, const uint64_t* fptr, const uint32_t* fids,
                                  uint32_t n_feat) {
    if (!c) return EP_ERR_INVALID_ARG;
    if (!fptr || (!fids && fptr[n_nodes])) return c->fail(EP_ERR_INVALID_ARG, "null feature arrays");
    if (n_nodes == 0 || n_nodes > 0xfffffffeull) return c->fail(EP_ERR_INVALID_ARG, "n_nodes must be in [1, 2^32-1)");
    if (c->graph_ok && n_nodes != c->n_nodes) return c->fail(EP_ERR_INVALID_ARG, "graph and features disagree on node count");
    if (n_feat == 0) return c->fail(EP_ERR_INVALID_ARG, "n_feat must be > 0");
    if (fptr[0] != 0) return c->fail(EP_ERR_INVALID_ARG, "features: row pointer must start at 0");
    cudaSetDevice(c->device);
    const uint64_t F = fptr[n_nodes];
    c->feats_ok = false;     // the device copy is replaced below; valid again once checked
    c->prepared = false;
    c->drop_graph();
    if (!c->fptr.ensure((n_nodes + 1) * 8) || !c->fids.ensure(F * 4)) return c->fail(EP_ERR_OOM, "feature allocation failed");
    CK(cudaMemcpyAsync(c->fptr.p, fptr, (n_nodes + 1) * 8, cudaMemcpyHostToDevice, c->stream), "upload fptr");
    if (F) CK(cudaMemcpyAsync(c->fids.p, fids, F * 4, cudaMemcpyHostToDevice, c->stream), "upload fids");
    uint32_t mx = 0;
    int rc = check_csr(c, n_nodes, c->fptr.as<uint64_t>(), c->fids.as<uint32_t>(), F, n_feat, "features", &mx);
    if (rc) return rc;
    if (c->table_ok && n_feat != c->n_feat) c->table_ok = false;
    c->n_nodes = n_nodes;
    c->n_fids = F;
    c->n_feat = n_feat;
    c->max_feat = mx;
    c->feats_ok = true;
    c->prepared = false;
    c->drop_graph();
    return EP_OK;
}

// Zeroes the Adam moments and restarts the pass sequence at pass 1, step 1.
static int reset_state(ep_ctx* c) {
    const size_t mv = (size_t)c->n_feat * c->dpad * sizeof(float);
    CK(cudaMemsetAsync(c->m.p, 0, mv, c->stream), "reset moments");
    CK(cudaMemsetAsync(c->v.p, 0, mv, c->stream), "reset moments");
    BatchState h{};
    h.pass = 1;
    h.batch = 0;
    h.step = 1;
    *c->h_st = h;
    if (!c->st.ensure(sizeof(BatchState)) || !c->st_eval.ensure(sizeof(BatchState)) || !c->st_inj.ensure(sizeof(BatchState)))
        return c->fail(EP_ERR_OOM, "state allocation failed");
    CK(cudaMemcpyAsync(c->st.p, c->h_st, sizeof(BatchState), cudaMemcpyHostToDevice, c->stream), "reset state");
    CK(cudaStreamSynchronize(c->stream), "reset state");
    c->host_pass = 1;
    c->host_batch = 0;
    c->state_ok = true;
    return EP_OK;
}

extern "C" int ep_set_table(ep_ctx* c, const float* init) {
    if (!c) return EP_ERR_INVALID_ARG;
    if (!c->feats_ok) return c->fail(EP_ERR_STATE, "upload features before setting the table");
    cudaSetDevice(c->device);
    const size_t es = c->tt == TT_BF16 ? 2 : 4;
    const size_t rows = (size_t)c->n_feat * c->dpad;
    if (!c->table.ensure(rows * es) || !c->m.ensure(rows * 4) || !c->v.ensure(rows * 4))
        return c->fail(EP_ERR_OOM, "table allocation failed (%zu rows)", (size_t)c->n_feat);
    if (init) {
        const size_t dense = (size_t)c->n_feat * c->dims * 4;
        if (!c->xfer.ensure(dense)) return c->fail(EP_ERR_OOM, "staging allocation failed");
        CK(cudaMemcpyAsync(c->xfer.p, init, dense, cudaMemcpyHostToDevice, c->stream), "upload table");
        launch_convert_table(c->tt, c->table.p, c->xfer.as<float>(), c->n_feat, c->dims, c->dpad, 1, c->stream);
    } else {
        launch_init_table(c->tt, c->table.p, c->n_feat, c->dims, c->dpad, c->cfg.seed, c->stream);
    }
    CK(cudaGetLastError(), "table init");
    c->table_ok = true;
    c->drop_graph();
    return reset_state(c);
}

extern "C" int ep_get_table(ep_ctx* c, float* out) {
    if (!c || !out) return EP_ERR_INVALID_ARG;
    if (!c->table_ok) return c->fail(EP_ERR_STATE, "no table");
    cudaSetDevice(c->device);
    // page-locked caller memory: the kernel writes the FP32 rows into it
    // directly (no staging buffer to allocate, no separate copy)
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, out) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer &&
        launch_table_out(c->tt, c->table.p, static_cast<float*>(pa.devicePointer), c->n_feat, c->dims, c->dpad,
                         c->stream)) {
        CK(cudaGetLastError(), "table download");
        CK(cudaStreamSynchronize(c->stream), "download table");
        return EP_OK;
    }
    cudaGetLastError();   // pageable memory: the attribute query may leave an error behind
    const size_t dense = (size_t)c->n_feat * c->dims * 4;
    if (!c->xfer.ensure(dense)) return c->fail(EP_ERR_OOM, "staging allocation failed");
    launch_convert_table(c->tt, c->table.p, c->xfer.as<float>(), c->n_feat, c->dims, c->dpad, 0, c->stream);
    CK(cudaGetLastError(), "table download");
    CK(cudaMemcpyAsync(out, c->xfer.p, dense, cudaMemcpyDeviceToHost, c->stream), "download table");
    CK(cudaStreamSynchronize(c->stream), "download table");
    return EP_OK;
}

// (Re)allocates per-batch scratch for B anchors, K neighbour slots, `items`
// gradient items and accumulator element size es.
static int ensure_bufs(ep_ctx* c, uint32_t B, uint32_t K, uint64_t items, uint32_t es, bool dense) {
    K = std::max<uint32_t>(K, 1);
    items = std::max<uint64_t>(items, 1);
    bool grow = B > c->buf_B || K > c->buf_K || items > c->items_cap || es > c->buf_es;
    if (grow) {
        B = std::max(B, c->buf_B);
        K = std::max(K, c->buf_K);
        items = std::max(items, c->items_cap);
        es = std::max(es, c->buf_es);
        const uint64_t NR = c->NR;
        const uint32_t nch = reduce_chunks(items, c->chunk);
        bool ok = c->anchors.ensure((size_t)B * 4) && c->nbr.ensure((size_t)B * K * 4) && c->nbr_w.ensure((size_t)B * K * 4) &&
                  c->nbr_cnt.ensure((size_t)B * 4) && c->neg.ensure((size_t)B * c->R * 4) && c->occ.ensure(((size_t)B + 1) * 4) &&
                  c->dir.ensure((size_t)B * NR * c->dpad * es) &&
                  (c->tt != TT_BF16 || c->dir16.ensure((size_t)B * NR * c->dpad * 2)) &&
                  c->scale.ensure((size_t)B * NR * es) &&
                  c->valid.ensure((size_t)B * NR) && c->loss.ensure((size_t)B * es) && c->status.ensure((size_t)B * 4) &&
                  c->deferred.ensure((size_t)B) &&
                  c->item_f.ensure(items * 4) && c->item_src.ensure(items * 4) && c->item_c.ensure(items * 4) &&
                  c->key_alt.ensure(items * 4) && c->idx.ensure(items * 8) && c->idx_alt.ensure(items * 8) &&
                  c->hist.ensure(radix_hist_entries(items) * 4) && c->carry_head.ensure((size_t)nch * c->dpad * es) &&
                  c->carry_tail.ensure((size_t)nch * c->dpad * es) && c->carry_f.ensure((size_t)nch * 4) &&
                  c->carry_flags.ensure((size_t)nch * 4) && c->long_list.ensure((size_t)nch * 8) &&
                  c->n_touched.ensure(4);
        if (!ok) return c->fail(EP_ERR_OOM, "batch scratch allocation failed (B=%u K=%u items=%llu)", B, K, (unsigned long long)items);
        c->buf_B = B;
        c->buf_K = K;
        c->long_cap = nch;
        c->items_cap = items;
        c->buf_es = es;
        c->drop_graph();
        // the sampling kernel reads nbr_cnt for every anchor slot
        CK(cudaMemsetAsync(c->nbr_cnt.p, 0, (size_t)B * 4, c->stream), "clear scratch");
    }
    if (dense) {
        const size_t rows = (size_t)c->n_feat * c->dpad * c->buf_es;
        const size_t tcap = (size_t)std::min<uint64_t>(c->n_feat, c->items_cap) * 4;
        if (!c->gdense.ensure(rows) || !c->touched.ensure(tcap)) return c->fail(EP_ERR_OOM, "dense gradient allocation failed");
    }
    return EP_OK;
}

static uint32_t feistel_half(uint64_t n) {
    const uint32_t b = bits_for(n);
    return (b + 1) / 2 ? (b + 1) / 2 : 1;
}

// Autotuner candidates: reducer chunk sizes (items per warp) and, for the
// FUSED form, the Adam placement (2: queued in the reducer, 1: split off).
constexpr uint32_t kTuneChunks[3] = {64, 128, 256};
constexpr uint32_t kTuneWarm = 2, kTuneTimed = 8;

// An upper bound of the sum of the `top` largest per-anchor item bounds,
// without copying the n bounds to the host: a 65,536-bin histogram of
// bound >> shift (count and sum per bin) is walked from the top; the bins
// taken whole add their exact sums, the partial bin its upper edge per
// anchor.  Exact when every bound is below 65,536.
__global__ void k_bound_max(const uint32_t* __restrict__ b, uint32_t n, uint32_t* mx) {
    uint32_t m = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = max(m, b[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(mx, m);
}

// Warp-aggregated: the lanes holding the same bin add once (their sum split
// into 16-bit halves so that 32 lanes cannot overflow a word).
__global__ void k_bound_hist(const uint32_t* __restrict__ b, uint32_t n, uint32_t shift, uint32_t* cnt,
                             unsigned long long* sum) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * blockDim.x / 32;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) / 32 * 32; base < n; base += warps * 32) {
        const uint32_t i = base + lane;
        const bool ok = i < n;                      // the whole warp iterates together
        const uint32_t x = ok ? b[i] : 0u;
        const uint32_t bin = ok ? x >> shift : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, bin);
        const uint32_t lo = __reduce_add_sync(peers, x & 0xffffu), hi = __reduce_add_sync(peers, x >> 16);
        if (ok && lane == __ffs(peers) - 1) {
            atomicAdd(&cnt[bin], (uint32_t)__popc(peers));
            atomicAdd(&sum[bin], ((unsigned long long)hi << 16) + lo);
        }
    }
}

static int top_sum_bound(ep_ctx* c, uint32_t n, uint32_t top, uint64_t* out) {
    constexpr uint32_t BINS = 65536;
    if (!c->check.ensure((size_t)BINS * 12 + 16)) return c->fail(EP_ERR_OOM, "scratch allocation failed");
    unsigned long long* sum = c->check.as<unsigned long long>();
    uint32_t* cnt = (uint32_t*)(sum + BINS);
    uint32_t* dmx = cnt + BINS;
    const uint32_t* b = c->bound.as<uint32_t>();
    CK(cudaMemsetAsync(c->check.p, 0, (size_t)BINS * 12 + 16, c->stream), "bounds");
    k_bound_max<<<152 * 4, 256, 0, c->stream>>>(b, n, dmx);
    uint32_t mx = 0;
    CK(cudaMemcpyAsync(&mx, dmx, 4, cudaMemcpyDeviceToHost, c->stream), "bounds");
    CK(cudaStreamSynchronize(c->stream), "bounds");
    uint32_t bits = 0;
    while (bits < 32 && (mx >> bits)) ++bits;
    const uint32_t shift = bits > 16 ? bits - 16 : 0;
    k_bound_hist<<<152 * 4, 256, 0, c->stream>>>(b, n, shift, cnt, sum);
    CK(cudaGetLastError(), "bounds");
    std::vector<uint32_t> hc(BINS);
    std::vector<unsigned long long> hs(BINS);
    CK(cudaMemcpyAsync(hc.data(), cnt, (size_t)BINS * 4, cudaMemcpyDeviceToHost, c->stream), "bounds");
    CK(cudaMemcpyAsync(hs.data(), sum, (size_t)BINS * 8, cudaMemcpyDeviceToHost, c->stream), "bounds");
    CK(cudaStreamSynchronize(c->stream), "bounds");
    uint64_t items = 0, left = top;
    for (int64_t bin = BINS - 1; bin >= 0 && left; --bin) {
        const uint64_t k = std::min<uint64_t>(hc[bin], left);
        if (k == hc[bin]) items += hs[bin];
        else items += k * ((((uint64_t)bin + 1) << shift) - 1);
        left -= k;
    }
    *out = items;
    return EP_OK;
}

static int prepare_train(ep_ctx* c) {
    if (!c->graph_ok || !c->feats_ok) return c->fail(EP_ERR_STATE, "upload the graph and the features first");
    if (!c->table_ok) return c->fail(EP_ERR_STATE, "set the table first");
    if (c->prepared) return EP_OK;
    const uint32_t n = (uint32_t)c->n_nodes;
    c->n_valid = (uint32_t)((float)n * c->cfg.valid_pct);   // mod.rs:121
    c->n_train = n - c->n_valid;
    if (c->n_train == 0) return c->fail(EP_ERR_INVALID_ARG, "no training nodes");
    if (!c->train_ids.ensure((size_t)c->n_train * 4) || !c->valid_ids.ensure((size_t)std::max<uint32_t>(c->n_valid, 1) * 4))
        return c->fail(EP_ERR_OOM, "id allocation failed");
    if (!c->st.ensure(sizeof(BatchState))) return c->fail(EP_ERR_OOM, "state allocation failed");
    // split: reuse the error word of the main state (cleared by reset_state)
    launch_split(c->train_ids.as<uint32_t>(), c->n_train, c->valid_ids.as<uint32_t>(), n, c->cfg.seed,
                 feistel_half(n), &c->st.as<BatchState>()->error, c->stream);
    const uint32_t B = c->cfg.batch_size;
    c->steps_per_pass = (uint32_t)((c->n_train + (uint64_t)B - 1) / B);
    const uint64_t steps_f = (uint64_t)ceilf((float)c->n_train / (float)B);   // mod.rs:125
    c->total_steps = steps_f * c->cfg.passes;
    c->warmup = (uint64_t)((float)c->total_steps / 5.f);                        // mod.rs:134
    uint32_t K = c->max_deg;
    if (c->cfg.max_nodes_kind == EP_SAMPLE_FIXED) K = std::min<uint32_t>((uint32_t)c->cfg.max_nodes, c->max_deg);
    if (c->cfg.loss == EP_LOSS_PPR) K = c->R;     // one slot per walk
    // item bound: sum of the B largest per-anchor bounds
    if (!c->bound.ensure((size_t)n * 4)) return c->fail(EP_ERR_OOM, "bound allocation failed");
    launch_node_bound(c->row.as<uint64_t>(), c->cols.as<uint32_t>(), c->fptr.as<uint64_t>(), n, c->cfg.max_nodes_kind,
                      (uint32_t)c->cfg.max_nodes, c->R, c->max_feat, c->cfg.loss == EP_LOSS_PPR,
                      c->bound.as<uint32_t>(), c->stream);
    uint64_t items = 0;
    int rcb = top_sum_bound(c, n, std::min<uint32_t>(B, n), &items);
    if (rcb) return rcb;
    if (items > 0xfffffff0ull) return c->fail(EP_ERR_UNSUPPORTED, "a batch can emit more than 2^32 gradient items");
    // with the autotuner, size the reducer carries for its smallest chunk and
    // keep the dense gradient buffers for the split Adam placement
    const uint32_t chunk = c->chunk;
    if (c->cfg.autotune >= 2) c->chunk = std::min<uint32_t>(c->chunk, kTuneChunks[0]);
    int rc = ensure_bufs(c, B, K, items, 4,
                         c->cfg.form == EP_FORM_PLAIN_FP32 || c->fused_mode == 1 || c->cfg.autotune >= 2);
    c->chunk = chunk;
    if (rc) return rc;
    c->Bcap = B;
    c->Kcap = c->buf_K;
    c->prepared = true;
    return EP_OK;
}

static FeatDrop feat_drop(const ep_ctx* c) {
    FeatDrop fd{};
    fd.kind = c->cfg.max_features_kind;
    fd.seed = c->cfg.seed;
    if (fd.kind == EP_SAMPLE_FIXED) fd.k = (uint32_t)c->cfg.max_features;
    if (fd.kind == EP_SAMPLE_PROB) {
        fd.p = c->cfg.max_features;
        const double t = (double)fd.p * 4294967296.0;
        fd.thr = t >= 4294967295.0 ? 0xffffffffu : (uint32_t)t;
    }
    return fd;
}

// Per-step decay of the gradient-noise scale: from cfg.noise at step 0 to
// 1e-9 after all updates (mod.rs:140-146), in f32 as the reference does.
static float noise_decay(const ep_ctx* c) {
    if (!(c->cfg.noise > 1e-9f) || c->total_steps == 0) return 1.f;
    const float min_noise = 1e-9f;
    return expf((logf(min_noise) - logf(c->cfg.noise)) / (float)c->total_steps);
}

static SampleParams sample_params(ep_ctx* c, BatchState* st, bool eval, int injected) {
    SampleParams sp{};
    sp.st = st;
    sp.cfg.nodes_kind = c->cfg.max_nodes_kind;
    sp.cfg.nodes_val = c->cfg.max_nodes;
    sp.cfg.K = (uint32_t)c->cfg.max_nodes;
    sp.cfg.Kcap = c->buf_K;
    sp.cfg.R = c->R;
    sp.cfg.weighted_avg = c->cfg.weighted_neighbor_averaging;
    sp.cfg.weighted_sampling = c->cfg.weighted_neighbor_sampling;
    sp.cfg.fd = feat_drop(c);
    sp.cfg.hard = c->cfg.hard_negatives;
    sp.cfg.ppr = c->cfg.loss == EP_LOSS_PPR;
    sp.cfg.ppr_restart = c->cfg.ppr_restart_p;
    sp.cfg.seed = c->cfg.seed;
    sp.row_ptr = c->row.as<uint64_t>();
    sp.cols = c->cols.as<uint32_t>();
    sp.wcdf = c->has_w ? c->wcdf.as<float>() : nullptr;
    sp.fptr = c->fptr.as<uint64_t>();
    sp.order = eval ? c->valid_ids.as<uint32_t>() : c->train_ids.as<uint32_t>();
    sp.n_order = eval ? c->n_valid : c->n_train;
    sp.pool = sp.order;
    sp.n_pool = sp.n_order;
    sp.batch_cap = injected ? c->buf_B : c->Bcap;
    sp.sample_warps = c->sample_warps;
    sp.injected = injected;
    sp.eval = eval;
    sp.feistel_half = feistel_half(sp.n_order);
    sp.anchors = c->anchors.as<uint32_t>();
    sp.nbr = c->nbr.as<uint32_t>();
    sp.nbr_w = c->nbr_w.as<float>();
    sp.nbr_cnt = c->nbr_cnt.as<uint32_t>();
    sp.neg = c->neg.as<uint32_t>();
    sp.occ = c->occ.as<uint32_t>();
    return sp;
}

static ForwardParams forward_params(ep_ctx* c, BatchState* st, const void* table, bool emit, bool eval) {
    ForwardParams fp{};
    fp.st = st;
    fp.loss = c->cfg.loss == EP_LOSS_PPR ? EP_LOSS_MARGIN : c->cfg.loss;   // PPR: margin on walk positives
    fp.gamma = c->cfg.gamma;
    fp.neg_margin = c->cfg.neg_margin;
    fp.loss_weighting = eval ? EP_LW_NONE : c->cfg.loss_weighting;   // validation reports the raw loss
    fp.lw_exp = c->cfg.loss_weighting_exp;
    fp.fd = feat_drop(c);
    fp.eval = eval;
    fp.R = c->R;
    fp.Kcap = c->buf_K;
    fp.dims = c->dims;
    fp.dpad = c->dpad;
    fp.row_ptr = c->row.as<uint64_t>();
    fp.fptr = c->fptr.as<uint64_t>();
    fp.fids = c->fids.as<uint32_t>();
    fp.table = table;
    fp.anchors = c->anchors.as<uint32_t>();
    fp.nbr = c->nbr.as<uint32_t>();
    fp.nbr_w = c->nbr_w.as<float>();
    fp.nbr_cnt = c->nbr_cnt.as<uint32_t>();
    fp.neg = c->neg.as<uint32_t>();
    fp.occ_off = c->occ.as<uint32_t>();
    fp.emit = emit;
    fp.items_cap = c->items_cap;
    fp.dir = c->dir.p;
    fp.dir16 = c->dir16.p;
    fp.scale = c->scale.p;
    fp.valid = c->valid.as<uint8_t>();
    fp.loss_out = c->loss.p;
    fp.status = c->status.as<int32_t>();
    fp.item_f = c->item_f.as<uint32_t>();
    fp.item_src = c->item_src.as<uint32_t>();
    fp.item_c = c->item_c.as<float>();
    fp.deferred = c->deferred.as<uint8_t>();
    fp.gather_ctas = c->gather_ctas;
    fp.gather_warps = c->gather_warps;
    return fp;
}

static ReduceParams reduce_params(ep_ctx* c, BatchState* st, int out_mode, void* table) {
    ReduceParams rp{};
    rp.st = st;
    rp.NR = c->NR;
    rp.dpad = c->dpad;
    rp.chunk = c->chunk;
    rp.grad_true = c->cfg.grad_mode == EP_GRAD_TRUE;
    rp.out_mode = out_mode;
    rp.skey = c->sorted_keys;
    rp.sval = c->sorted_vals;
    rp.dir = c->dir.p;
    rp.dir16 = c->dir16.p;
    rp.scale = c->scale.p;
    rp.valid = c->valid.as<uint8_t>();
    rp.table = table;
    rp.m = c->m.as<float>();
    rp.v = c->v.as<float>();
    rp.seed = c->cfg.seed;
    rp.gdense = c->gdense.p;
    rp.touched = c->touched.as<uint32_t>();
    rp.n_touched = c->n_touched.as<uint32_t>();
    rp.carry_head = c->carry_head.p;
    rp.carry_tail = c->carry_tail.p;
    rp.carry_f = c->carry_f.as<uint32_t>();
    rp.carry_flags = c->carry_flags.as<uint32_t>();
    rp.long_list = c->long_list.as<uint32_t>();
    rp.long_cap = c->long_cap;
    rp.ring_pw = c->ring_pw;
    rp.ring_cw = c->ring_cw;
    rp.ring_slots = c->ring_slots;
    rp.queue_ctas_per_sm = c->queue_ctas;
    rp.red_ctas = c->red_ctas;
    return rp;
}

// Sort the emitted items and reduce them; tt selects the kernel family.
static void sort_and_reduce(ep_ctx* c, BatchState* st, int tt, int out_mode, void* table, cudaStream_t s) {
    launch_radix_sort(st, c->item_f.as<uint32_t>(), c->key_alt.as<uint32_t>(), c->item_src.as<uint32_t>(),
                      c->item_c.as<float>(), c->idx.as<uint2>(), c->idx_alt.as<uint2>(), c->hist.as<uint32_t>(),
                      c->items_cap, (int)bits_for(c->n_feat), &c->sorted_keys, &c->sorted_vals, s);
    if (out_mode == OUT_DENSE) cudaMemsetAsync(c->n_touched.p, 0, 4, s);
    ReduceParams rp = reduce_params(c, st, out_mode, table);
    launch_reduce(tt, (int)c->vpl, rp, c->items_cap, s);
    launch_fixup(tt, (int)c->vpl, rp, c->items_cap, s);
}

// The FUSED form's reduction output for its Adam placement (fused_mode 0,
// 2, 3); the ring falls back to the per-warp queue for row shapes it cannot
// bulk-copy.
static int fused_out_mode(const ep_ctx* c) {
    if (c->fused_mode == 3)
        return ring_supported(c->tt, c->dpad, c->ring_pw, c->ring_cw, c->ring_slots) ? OUT_RING : OUT_QUEUE;
    return c->fused_mode == 2 ? OUT_QUEUE : OUT_ADAM;
}

// Kernels launched per training batch.
static uint32_t kernels_per_batch(const ep_ctx* c, bool fork) {
    const uint32_t b = bits_for(c->n_feat);
    const uint32_t radix = 3 * (b ? (b + 7) / 8 : 1);
    return 3 /* begin, sample, scan */ + 3 /* forward: staged, direct gather; loss */ + (fork ? 1 : 0) /* emit */ + radix +
           3 /* reduce, fixup x2 */ +
           (c->cfg.form == EP_FORM_PLAIN_FP32 || c->fused_mode == 1 ? 1 : 0) + 1 /* end */;
}

// Issues one training batch on the context stream; ev (optional) receives an
// event record after each stage (EP_N_STAGES events).  With fork (graph
// capture), the item offsets are scanned, the items emitted by k_fwd_emit and
// sorted on the side stream beside the gathers and the loss (which then skip
// the emission and read neither), and k_batch_end follows the loss there; the
// reduction waits for the sorted items.  The fix-ups run on the fix stream
// beside the next batch's k_batch_begin, sampler and scan (which read neither
// the table nor what the fix-ups read: those use k_reduce's copy of the item
// count and Adam constants), and that batch's gathers and item emission wait
// for them; the last batch of a capture (last) joins its fix-ups before it
// ends.
static void issue_train_batch(ep_ctx* c, cudaEvent_t* ev = nullptr, bool fork = false, bool last = true) {
    BatchState* st = c->st.as<BatchState>();
    cudaStream_t s = c->stream;
    launch_batch_begin(st, c->n_train, c->Bcap, c->steps_per_pass, c->total_steps, c->warmup, c->cfg.alpha, 0,
                       c->cfg.noise, noise_decay(c), s);
    SampleParams sp = sample_params(c, st, false, false);
    launch_sample(sp, s);
    if (!fork) launch_scan_occ(st, c->occ.as<uint32_t>(), c->Bcap, c->items_cap, s);
    if (ev) cudaEventRecord(ev[EP_STAGE_SAMPLE], s);
    if (fork) {
        // side stream: the item offsets (scan), the items (k_fwd_emit) and
        // their sort, beside the gathers and the loss on the main stream,
        // which run with emission off and read neither; then k_batch_end
        cudaEventRecord(c->ev_fork, s);
        cudaStreamWaitEvent(c->side, c->ev_fork, 0);
        launch_scan_occ(st, c->occ.as<uint32_t>(), c->Bcap, c->items_cap, c->side);
        if (c->fix_pending) {   // the previous batch's fix-ups: the table, and the sorted items they read
            cudaStreamWaitEvent(s, c->ev_fix, 0);
            cudaStreamWaitEvent(s, c->ev_fix2, 0);
            cudaStreamWaitEvent(c->side, c->ev_fix, 0);
            cudaStreamWaitEvent(c->side, c->ev_fix2, 0);
            c->fix_pending = false;
        }
        ForwardParams fe = forward_params(c, st, c->table.p, true, false);
        launch_forward(c->tt, (int)c->vpl, fe, c->Bcap, c->side, FWD_EMIT);
        launch_radix_sort(st, c->item_f.as<uint32_t>(), c->key_alt.as<uint32_t>(), c->item_src.as<uint32_t>(),
                          c->item_c.as<float>(), c->idx.as<uint2>(), c->idx_alt.as<uint2>(), c->hist.as<uint32_t>(),
                          c->items_cap, (int)bits_for(c->n_feat), &c->sorted_keys, &c->sorted_vals, c->side);
        cudaEventRecord(c->ev_sorted, c->side);
        ForwardParams fp = forward_params(c, st, c->table.p, false, false);
        fp.means_dead = 1;
        launch_forward(c->tt, (int)c->vpl, fp, c->Bcap, s);
        cudaEventRecord(c->ev_loss, s);
        cudaStreamWaitEvent(c->side, c->ev_loss, 0);
        launch_batch_end(st, c->loss.p, c->status.as<int32_t>(), c->nbr_cnt.as<uint32_t>(), c->Bcap, c->steps_per_pass,
                         0, 0, c->side);
        cudaEventRecord(c->ev_join, c->side);
        cudaStreamWaitEvent(s, c->ev_sorted, 0);   // sorted items for the reduction
    } else {
        ForwardParams fp = forward_params(c, st, c->table.p, true, false);
        fp.means_dead = 1;
        launch_forward(c->tt, (int)c->vpl, fp, c->Bcap, s);
        if (ev) cudaEventRecord(ev[EP_STAGE_FORWARD], s);
        launch_radix_sort(st, c->item_f.as<uint32_t>(), c->key_alt.as<uint32_t>(), c->item_src.as<uint32_t>(),
                          c->item_c.as<float>(), c->idx.as<uint2>(), c->idx_alt.as<uint2>(), c->hist.as<uint32_t>(),
                          c->items_cap, (int)bits_for(c->n_feat), &c->sorted_keys, &c->sorted_vals, s);
        if (ev) cudaEventRecord(ev[EP_STAGE_SORT], s);
    }
    const bool plain = c->cfg.form == EP_FORM_PLAIN_FP32 || c->fused_mode == 1;
    if (plain) cudaMemsetAsync(c->n_touched.p, 0, 4, s);
    ReduceParams rp = reduce_params(c, st, plain ? OUT_DENSE : fused_out_mode(c), c->table.p);
    launch_reduce(c->tt, (int)c->vpl, rp, c->items_cap, s);
    if (ev) cudaEventRecord(ev[EP_STAGE_REDUCE], s);
    if (fork && !plain) {
        cudaEventRecord(c->ev_red, s);
        cudaStreamWaitEvent(c->fix, c->ev_red, 0);
        cudaStreamWaitEvent(c->fix2, c->ev_red, 0);
        launch_fixup(c->tt, (int)c->vpl, rp, c->items_cap, c->fix, 1);    // short spans
        launch_fixup(c->tt, (int)c->vpl, rp, c->items_cap, c->fix2, 2);   // long spans, beside them
        cudaEventRecord(c->ev_fix, c->fix);
        cudaEventRecord(c->ev_fix2, c->fix2);
        if (last) {
            cudaStreamWaitEvent(s, c->ev_fix, 0);
            cudaStreamWaitEvent(s, c->ev_fix2, 0);
        } else {
            c->fix_pending = true;
        }
    } else {
        // the long spans' fix-ups beside the short ones here too
        cudaEventRecord(c->ev_red, s);
        cudaStreamWaitEvent(c->fix2, c->ev_red, 0);
        launch_fixup(c->tt, (int)c->vpl, rp, c->items_cap, s, 1);
        launch_fixup(c->tt, (int)c->vpl, rp, c->items_cap, c->fix2, 2);
        cudaEventRecord(c->ev_fix2, c->fix2);
        cudaStreamWaitEvent(s, c->ev_fix2, 0);
    }
    if (ev) cudaEventRecord(ev[EP_STAGE_FIXUP], s);
    if (plain)
        launch_adam_dense(c->tt, (int)c->vpl, st, c->table.p, c->m.as<float>(), c->v.as<float>(), c->gdense.as<float>(),
                          c->touched.as<uint32_t>(), c->n_touched.as<uint32_t>(), c->dpad,
                          (uint32_t)std::min<uint64_t>(c->n_feat, c->items_cap), c->cfg.seed, s);
    if (ev) cudaEventRecord(ev[EP_STAGE_ADAM], s);
    if (fork) cudaStreamWaitEvent(s, c->ev_join, 0);
    else launch_batch_end(st, c->loss.p, c->status.as<int32_t>(), c->nbr_cnt.as<uint32_t>(), c->Bcap, c->steps_per_pass, 0, 0, s);
    if (ev) cudaEventRecord(ev[EP_STAGE_END], s);
    c->launches += kernels_per_batch(c, fork);
}

static void advance_host_batch(ep_ctx* c) {
    if (++c->host_batch >= c->steps_per_pass) { c->host_batch = 0; ++c->host_pass; }
}

static int launch_train_batch(ep_ctx* c);

// Issues n consecutive training batches.  With graphs, runs of graph_batches
// batches replay one graph holding that many copies of the batch (the
// device-resident BatchState moves each copy to the next batch, crossing pass
// boundaries as the device would); a remainder of r >= 2 batches replays a
// graph of r batches, a single batch the one-batch graph.
//
// The autotuner (config.autotune) times kTuneTimed batches after kTuneWarm
// warm-up batches under each candidate launch shape and keeps the fastest.
// Level 1 tries only shapes that leave every result bit-identical (tested):
// the FUSED form's Adam placement -- queued in the reducing warp, or the
// warp-specialised ring with two splits of a CTA into reducing and Adam
// warps -- and the staged gather's grid: one warp per anchor, or a persistent
// grid of 2 or 3 CTAs per SM taking anchors from a work queue.  Level 2 also
// tries reducer chunk sizes and the split-off Adam kernel; chunk sizes change
// the floating-point summation order, so level 2 trades reproducibility for
// speed.  The batches it runs are ordinary training batches of the pass (they
// update the table); it runs once per context, when at least all candidates'
// batches are requested in one call, and its choice is remembered per
// workload shape and device, so later contexts on the same shape start with
// it.  Chosen values: ep_get_tuning, ep_get_launch_shape.
struct TuneChoice {
    uint32_t chunk;
    int mode;
    uint32_t gather_ctas, pw, cw, slots, qctas, gwarps;
};

namespace {
std::mutex g_tune_mu;
std::map<std::vector<uint64_t>, TuneChoice> g_tune_cache;

std::vector<uint64_t> tune_key(const ep_ctx* c) {
    return {(uint64_t)c->cfg.form, (uint64_t)c->cfg.autotune, c->dims, c->Bcap, c->R, c->Kcap, c->n_feat, c->n_nodes,
            c->n_edges, (uint64_t)c->cfg.loss, (uint64_t)c->device, (uint64_t)c->cfg.max_features_kind};
}

void apply_choice(ep_ctx* c, const TuneChoice& t) {
    c->chunk = t.chunk;
    c->fused_mode = t.mode;
    c->gather_ctas = t.gather_ctas;
    c->ring_pw = t.pw;
    c->ring_cw = t.cw;
    c->ring_slots = t.slots;
    c->queue_ctas = t.qctas;
    c->gather_warps = t.gwarps;
    c->drop_graph();
}
}  // namespace

// Times each candidate on real batches; returns the fastest (or the current
// shape when a launch fails, with rc set).
static int tune_stage(ep_ctx* c, const std::vector<TuneChoice>& cands, TuneChoice* pick) {
    if (cands.size() < 2) {
        if (!cands.empty()) *pick = cands[0];
        return EP_OK;
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "tuning events");
    CK(cudaEventCreate(&e1), "tuning events");
    float best = 0.f;
    int rc = EP_OK;
    for (size_t i = 0; i < cands.size() && !rc; ++i) {
        apply_choice(c, cands[i]);
        for (uint32_t b = 0; b < kTuneWarm && !rc; ++b) rc = launch_train_batch(c);
        cudaEventRecord(e0, c->stream);
        for (uint32_t b = 0; b < kTuneTimed && !rc; ++b) rc = launch_train_batch(c);
        cudaEventRecord(e1, c->stream);
        if (rc) break;
        if (cudaEventSynchronize(e1) != cudaSuccess) { rc = c->cuda_fail(cudaGetLastError(), "tuning"); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (i == 0 || ms < best) { best = ms; *pick = cands[i]; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

// A choice remembered for this workload shape, applied without timing.
static bool tune_from_cache(ep_ctx* c) {
    if (!c->cfg.autotune || c->tuned) return c->tuned;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(tune_key(c));
    if (it == g_tune_cache.end()) return false;
    apply_choice(c, it->second);
    c->tuned = true;
    return true;
}

// Candidates of the two tuning stages; `need` receives the batches they take.
static void tune_candidates(const ep_ctx* c, std::vector<TuneChoice>& s1, uint32_t& need) {
    const TuneChoice cur = {c->chunk, c->fused_mode, c->gather_ctas, c->ring_pw, c->ring_cw, c->ring_slots, c->queue_ctas,
                           c->gather_warps};
    const bool fused = c->cfg.form == EP_FORM_FUSED_BF16;
    const int level = c->cfg.autotune;
    // stage 1: reducer chunk (level 2) x Adam placement (FUSED form)
    const std::vector<uint32_t> chunks = level >= 2 ? std::vector<uint32_t>(kTuneChunks, kTuneChunks + 3)
                                                    : std::vector<uint32_t>{c->chunk};
    for (uint32_t ch : chunks) {
        TuneChoice t = cur;
        t.chunk = ch;
        if (!fused) { s1.push_back(t); continue; }
        t.mode = 2;
        t.qctas = 4;
        s1.push_back(t);
        if (c->vpl <= 8) { t.qctas = 5; s1.push_back(t); t.qctas = 4; }
        if (level >= 2) { t.mode = 1; s1.push_back(t); }
        const uint32_t rings[2][3] = {{12, 4, 32}, {10, 6, 36}};
        for (const auto& r : rings)
            if (ring_supported(c->tt, c->dpad, r[0], r[1], r[2])) {
                t.mode = 3; t.pw = r[0]; t.cw = r[1]; t.slots = r[2];
                s1.push_back(t);
            }
    }
    // stage 2 times five gather grids
    need = (uint32_t)((s1.size() > 1 ? s1.size() : 0) + 5) * (kTuneWarm + kTuneTimed);
}

static int autotune(ep_ctx* c, uint32_t& n) {
    if (tune_from_cache(c)) return EP_OK;
    const TuneChoice cur = {c->chunk, c->fused_mode, c->gather_ctas, c->ring_pw, c->ring_cw, c->ring_slots, c->queue_ctas,
                           c->gather_warps};
    std::vector<TuneChoice> s1;
    uint32_t need = 0;
    tune_candidates(c, s1, need);
    if (n < need) return EP_OK;
    // stage 2: the staged gather's grid, with the stage-1 choice: one warp per
    // anchor in CTAs of 2, 4 or 8 warps, or persistent at 2 or 3 CTAs per SM
    const uint32_t gathers[5][2] = {{0, 2}, {0, 4}, {0, 8}, {2 * 152, 8}, {3 * 152, 8}};
    TuneChoice pick = cur;
    int rc = tune_stage(c, s1, &pick);
    std::vector<TuneChoice> s2;
    for (const auto& g : gathers) {
        TuneChoice t = pick;
        t.gather_ctas = g[0];
        t.gwarps = g[1];
        s2.push_back(t);
    }
    if (!rc) rc = tune_stage(c, s2, &pick);
    if (rc) {
        apply_choice(c, cur);
        return rc;
    }
    n -= need;
    apply_choice(c, pick);
    c->tuned = true;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[tune_key(c)] = pick;
    return EP_OK;
}

// Captures, instantiates and uploads `batches` consecutive training batches
// as one graph (nothing runs: the capture only records the launches).
static int capture_batches(ep_ctx* c, uint32_t batches, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
    const uint64_t before = c->launches;
    for (uint32_t i = 0; i < batches; ++i) issue_train_batch(c, nullptr, true, i + 1 == batches);
    c->launches = before;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) return c->cuda_fail(e, "graph capture");
    e = cudaGraphInstantiate(out, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { *out = nullptr; return c->cuda_fail(e, "graph instantiate"); }
    // the graph's work goes to the device now, not at its first launch
    e = cudaGraphUpload(*out, c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "graph upload");
    return EP_OK;
}

// Builds, ahead of a run of n batches, the graphs that run will replay, so
// that the one-time capture and instantiation stay outside its timing.
static int prepare_graphs(ep_ctx* c, uint32_t n) {
    if (!(c->cfg.use_graphs && c->cfg.form == EP_FORM_FUSED_BF16) || n == 0) return EP_OK;
    if (c->cfg.autotune && !tune_from_cache(c)) {
        std::vector<TuneChoice> s1;
        uint32_t need = 0;
        tune_candidates(c, s1, need);
        if (n >= need) return EP_OK;   // this run starts with the tuner, which rebuilds them per candidate
    }
    const uint32_t k = c->graph_batches;
    int rc = EP_OK;
    if (k > 1 && n >= k && !c->gexec_run) rc = capture_batches(c, k, &c->gexec_run);
    const uint32_t r = k > 1 ? n % k : 1;
    if (!rc && r == 1 && !c->gexec) rc = capture_batches(c, 1, &c->gexec);
    if (!rc && r >= 2 && !c->gexec_rem.count(r)) {
        cudaGraphExec_t g = nullptr;
        rc = capture_batches(c, r, &g);
        if (!rc) c->gexec_rem[r] = g;
    }
    return rc;
}

static int launch_train_run(ep_ctx* c, uint32_t n) {
    if (c->cfg.autotune && !c->tuned) {
        int rc = autotune(c, n);
        if (rc) return rc;
    }
    const bool use_graph = c->cfg.use_graphs && c->cfg.form == EP_FORM_FUSED_BF16;
    const uint32_t k = c->graph_batches;
    while (n) {
        if (use_graph && k > 1 && n >= k) {
            if (!c->gexec_run) {
                int rc = capture_batches(c, k, &c->gexec_run);
                if (rc) return rc;
            }
            CK(cudaGraphLaunch(c->gexec_run, c->stream), "graph launch");
            c->launches += (uint64_t)k * kernels_per_batch(c, true);
            for (uint32_t i = 0; i < k; ++i) advance_host_batch(c);
            n -= k;
        } else if (use_graph && n >= 2) {
            // the run's remainder as one graph of n batches: their fix-ups
            // overlap the next batch's sampling as in the full-size graph
            auto it = c->gexec_rem.find(n);
            if (it == c->gexec_rem.end()) {
                cudaGraphExec_t g = nullptr;
                int rc = capture_batches(c, n, &g);
                if (rc) return rc;
                it = c->gexec_rem.emplace(n, g).first;
            }
            CK(cudaGraphLaunch(it->second, c->stream), "graph launch");
            c->launches += (uint64_t)n * kernels_per_batch(c, true);
            for (uint32_t i = 0; i < n; ++i) advance_host_batch(c);
            n = 0;
        } else {
            int rc = launch_train_batch(c);
            if (rc) return rc;
            --n;
        }
    }
    return EP_OK;
}

static int launch_train_batch(ep_ctx* c) {
    const bool use_graph = c->cfg.use_graphs && c->cfg.form == EP_FORM_FUSED_BF16;
    if (use_graph) {
        if (!c->gexec) {
            int rc = capture_batches(c, 1, &c->gexec);
            if (rc) return rc;
        }
        CK(cudaGraphLaunch(c->gexec, c->stream), "graph launch");
        c->launches += kernels_per_batch(c, true);
    } else {
        issue_train_batch(c);
        CK(cudaGetLastError(), "batch launch");
    }
    advance_host_batch(c);
    return EP_OK;
}

// Validation pass over the held-out ids (mod.rs:267-283): forward only, fixed
// sampling stream, negatives from the validation ids.
static int run_validation(ep_ctx* c, double* mean_out) {
    *mean_out = NAN;
    if (c->n_valid == 0) return EP_OK;
    BatchState h{};
    h.pass = 1;
    h.step = 1;
    BatchState* st = c->st_eval.as<BatchState>();
    CK(cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream), "eval state");
    const uint32_t nb = (c->n_valid + c->Bcap - 1) / c->Bcap;
    for (uint32_t b = 0; b < nb; ++b) {
        launch_batch_begin(st, c->n_valid, c->Bcap, nb, 1, 0, c->cfg.alpha, 0, 0.f, 1.f, c->stream);
        SampleParams sp = sample_params(c, st, true, false);
        launch_sample(sp, c->stream);
        ForwardParams fp = forward_params(c, st, c->table.p, false, true);
        launch_forward(c->tt, (int)c->vpl, fp, c->Bcap, c->stream);
        launch_batch_end(st, c->loss.p, c->status.as<int32_t>(), c->nbr_cnt.as<uint32_t>(), c->Bcap, nb, 1, 0, c->stream);
    }
    CK(cudaGetLastError(), "validation launch");
    CK(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, c->stream), "eval state");
    CK(cudaStreamSynchronize(c->stream), "validation");
    *mean_out = h.valid_sum / (double)c->n_valid;
    return EP_OK;
}

static int clear_accumulators(ep_ctx* c) {
    c->launches = 0;
    const size_t off = offsetof(BatchState, pass_err_sum);
    CK(cudaMemsetAsync((char*)c->st.p + off, 0, sizeof(BatchState) - off, c->stream), "clear counters");
    return EP_OK;
}

static int read_state(ep_ctx* c) {
    CK(cudaMemcpyAsync(c->h_st, c->st.p, sizeof(BatchState), cudaMemcpyDeviceToHost, c->stream), "read state");
    CK(cudaStreamSynchronize(c->stream), "batch execution");
    if (c->h_st->error) return c->fail(EP_ERR_DEVICE, "device error flags 0x%x", c->h_st->error);
    return EP_OK;
}

static void fill_stats(ep_ctx* c, ep_pass_stats* s, uint32_t pass, double ms, double valid) {
    const BatchState& h = *c->h_st;
    memset(s, 0, sizeof(*s));
    s->pass = pass;
    s->batches = h.pass_batches;
    s->train_loss = h.pass_batches ? (float)(h.pass_err_sum / (double)h.pass_batches) : 0.f;
    s->valid_loss = (float)valid;
    s->lr_last = h.lr;
    s->noise_last = h.noise_sigma;
    s->anchors = h.anchors;
    s->kept_anchors = h.kept;
    s->nan_anchors = h.nan_anchors;
    s->items = h.items;
    s->gathered_rows = h.gathered;
    s->unique_rows = h.unique_rows;
    s->sampled_neighbors = h.sampled;
    s->ms = ms;
    const double d = c->dims, es = c->tt == TT_BF16 ? 2.0 : 4.0;
    s->alg_bytes = (double)h.gathered * d * es + (double)h.unique_rows * d * (2 * es + 16) + 4.0 * h.gathered +
                   4.0 * h.sampled + 8.0 * (double)h.anchors * (c->R + 2);
    s->launches = c->launches;
}

extern "C" int ep_train(ep_ctx* c, ep_pass_stats* stats, uint32_t stats_len) {
    if (!c) return EP_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    int rc = prepare_train(c);
    if (rc) return rc;
    rc = reset_state(c);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (uint32_t pass = 1; pass <= c->cfg.passes; ++pass) {
        if ((rc = clear_accumulators(c))) break;
        if ((rc = prepare_graphs(c, c->steps_per_pass))) break;
        cudaEventRecord(e0, c->stream);
        if ((rc = launch_train_run(c, c->steps_per_pass))) break;
        cudaEventRecord(e1, c->stream);
        if ((rc = read_state(c))) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        double valid = NAN;
        if ((rc = run_validation(c, &valid))) break;
        if (stats && pass <= stats_len) fill_stats(c, &stats[pass - 1], pass, ms, valid);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

extern "C" int ep_train_batches(ep_ctx* c, uint32_t n_batches, ep_pass_stats* stats) {
    if (!c) return EP_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    int rc = prepare_train(c);
    if (rc) return rc;
    if (!c->state_ok && (rc = reset_state(c))) return rc;
    if ((rc = clear_accumulators(c))) return rc;
    if ((rc = prepare_graphs(c, n_batches))) return rc;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, c->stream);
    rc = launch_train_run(c, n_batches);
    cudaEventRecord(e1, c->stream);
    if (!rc) rc = read_state(c);
    float ms = 0.f;
    if (!rc) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc && stats) fill_stats(c, stats, c->host_pass, ms, NAN);
    return rc;
}

extern "C" int ep_profile_batches(ep_ctx* c, uint32_t n_batches, double* stage_ms, ep_pass_stats* stats) {
    if (!c || !stage_ms) return EP_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    int rc = prepare_train(c);
    if (rc) return rc;
    if (!c->state_ok && (rc = reset_state(c))) return rc;
    if ((rc = clear_accumulators(c))) return rc;
    std::vector<cudaEvent_t> ev((size_t)n_batches * EP_N_STAGES + 1);
    for (auto& e : ev) cudaEventCreate(&e);
    cudaEventRecord(ev[0], c->stream);
    for (uint32_t b = 0; b < n_batches; ++b) {
        issue_train_batch(c, &ev[1 + (size_t)b * EP_N_STAGES]);
        if (++c->host_batch >= c->steps_per_pass) { c->host_batch = 0; ++c->host_pass; }
    }
    rc = read_state(c);
    for (int k = 0; k < EP_N_STAGES; ++k) stage_ms[k] = 0.0;
    double total = 0.0;
    if (!rc) {
        for (uint32_t b = 0; b < n_batches; ++b)
            for (int k = 0; k < EP_N_STAGES; ++k) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev[(size_t)b * EP_N_STAGES + k], ev[1 + (size_t)b * EP_N_STAGES + k]);
                stage_ms[k] += ms;
                total += ms;
            }
        for (int k = 0; k < EP_N_STAGES; ++k) stage_ms[k] /= n_batches ? n_batches : 1;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (!rc && stats) fill_stats(c, stats, c->host_pass, total, NAN);
    return rc;
}

extern "C" int ep_synchronize(ep_ctx* c) {
    if (!c) return EP_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    CK(cudaStreamSynchronize(c->stream), "synchronize");
    if (c->state_ok) return read_state(c);
    return EP_OK;
}

// ---------------------------------------------------------------------------
// Explicit-sample paths (parity hooks and the autograd binding)
// ---------------------------------------------------------------------------
static int stage_samples(ep_ctx* c, const ep_batch_samples* sm, uint32_t es, cudaStream_t s) {
    if (!sm || !sm->anchors || !sm->nbr_ptr || !sm->negatives) return c->fail(EP_ERR_INVALID_ARG, "null sample arrays");
    if (!c->graph_ok || !c->feats_ok) return c->fail(EP_ERR_STATE, "upload the graph and the features first");
    const uint32_t B = sm->n_anchors;
    if (B == 0) return c->fail(EP_ERR_INVALID_ARG, "empty batch");
    uint32_t K = 1;
    for (uint32_t a = 0; a < B; ++a) {
        if (sm->nbr_ptr[a + 1] < sm->nbr_ptr[a]) return c->fail(EP_ERR_INVALID_ARG, "nbr_ptr decreases at %u", a);
        K = std::max(K, sm->nbr_ptr[a + 1] - sm->nbr_ptr[a]);
        if (sm->anchors[a] >= c->n_nodes) return c->fail(EP_ERR_INVALID_ARG, "anchor id out of range");
    }
    const uint32_t nn = sm->nbr_ptr[B];
    if (nn && (!sm->nbr || !sm->nbr_w)) return c->fail(EP_ERR_INVALID_ARG, "null neighbour arrays");
    for (uint32_t j = 0; j < nn; ++j)
        if (sm->nbr[j] >= c->n_nodes) return c->fail(EP_ERR_INVALID_ARG, "neighbour id out of range");
    for (uint64_t j = 0; j < (uint64_t)B * c->R; ++j)
        if (sm->negatives[j] >= c->n_nodes) return c->fail(EP_ERR_INVALID_ARG, "negative id out of range");
    const uint64_t items = (uint64_t)B * c->max_feat * (1ull + c->R + K);
    int rc = ensure_bufs(c, B, K, items, es, true);
    if (rc) return rc;
    const uint32_t Ks = c->buf_K;
    std::vector<uint32_t> nb((size_t)B * Ks, 0u), cnt(B);
    std::vector<float> nw((size_t)B * Ks, 0.f);
    for (uint32_t a = 0; a < B; ++a) {
        cnt[a] = sm->nbr_ptr[a + 1] - sm->nbr_ptr[a];
        for (uint32_t j = 0; j < cnt[a]; ++j) {
            nb[(size_t)a * Ks + j] = sm->nbr[sm->nbr_ptr[a] + j];
            nw[(size_t)a * Ks + j] = sm->nbr_w[sm->nbr_ptr[a] + j];
        }
    }
    CK(cudaMemcpyAsync(c->anchors.p, sm->anchors, (size_t)B * 4, cudaMemcpyHostToDevice, s), "stage anchors");
    CK(cudaMemcpyAsync(c->nbr.p, nb.data(), nb.size() * 4, cudaMemcpyHostToDevice, s), "stage neighbours");
    CK(cudaMemcpyAsync(c->nbr_w.p, nw.data(), nw.size() * 4, cudaMemcpyHostToDevice, s), "stage weights");
    CK(cudaMemcpyAsync(c->nbr_cnt.p, cnt.data(), (size_t)B * 4, cudaMemcpyHostToDevice, s), "stage counts");
    CK(cudaMemcpyAsync(c->neg.p, sm->negatives, (size_t)B * c->R * 4, cudaMemcpyHostToDevice, s), "stage negatives");
    CK(cudaStreamSynchronize(s), "stage samples");   // host vectors go out of scope
    return EP_OK;
}

// Runs count -> scan -> forward -> sort -> reduce for staged samples.
static int run_injected(ep_ctx* c, uint32_t B, int tt, const void* table, void* loss_out, const void* dloss,
                        int out_mode, void* adam_table, float lr, uint32_t pass, cudaStream_t s) {
    BatchState h{};
    h.pass = pass;
    h.step = 1;
    h.n_anchors = B;
    h.lr = lr;
    h.bc1 = 1.f - powf(0.9f, (float)pass + 1.f);
    h.bc2 = 1.f - powf(0.999f, (float)pass + 1.f);
    h.noise_sigma = c->cfg.noise > 1e-9f ? c->cfg.noise : 0.f;   // injected steps: the configured scale
    BatchState* st = c->st_inj.as<BatchState>();
    if (!c->st_inj.ensure(sizeof(BatchState))) return c->fail(EP_ERR_OOM, "state allocation failed");
    st = c->st_inj.as<BatchState>();
    CK(cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s), "inject state");
    SampleParams sp = sample_params(c, st, false, true);
    launch_sample(sp, s);
    launch_scan_occ(st, c->occ.as<uint32_t>(), B, c->items_cap, s);
    ForwardParams fp = forward_params(c, st, table, true, false);
    fp.loss_out = loss_out;
    fp.dloss = (const float*)dloss;
    fp.dloss_f64 = tt == TT_F64;
    launch_forward(tt, (int)c->vpl, fp, B, s);
    sort_and_reduce(c, st, tt, out_mode, adam_table, s);
    if (out_mode == OUT_DENSE && adam_table)
        launch_adam_dense(tt, (int)c->vpl, st, adam_table, c->m.as<float>(), c->v.as<float>(), c->gdense.as<float>(),
                          c->touched.as<uint32_t>(), c->n_touched.as<uint32_t>(), c->dpad,
                          (uint32_t)std::min<uint64_t>(c->n_feat, c->items_cap), c->cfg.seed, s);
    CK(cudaGetLastError(), "injected batch launch");
    CK(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s), "read state");
    CK(cudaStreamSynchronize(s), "injected batch");
    if (h.error) return c->fail(EP_ERR_DEVICE, "device error flags 0x%x", h.error);
    return EP_OK;
}

extern "C" int ep_sample(ep_ctx* c, const uint32_t* anchors, uint32_t n, uint32_t step, uint32_t stride,
                         uint32_t* nbr_cnt, uint32_t* nbr, float* nbr_w, uint32_t* neg) {
    if (!c) return EP_ERR_INVALID_ARG;
    if (n && (!anchors || !nbr_cnt || !nbr || !nbr_w || !neg)) return c->fail(EP_ERR_INVALID_ARG, "null array");
    cudaSetDevice(c->device);
    int rc = prepare_train(c);
    if (rc) return rc;
    if (n > c->Bcap) return c->fail(EP_ERR_INVALID_ARG, "%u anchors exceed the batch size %u", n, c->Bcap);
    if (stride < c->Kcap)
        return c->fail(EP_ERR_INVALID_ARG, "neighbour stride %u below the %u slots an anchor can fill", stride, c->Kcap);
    for (uint32_t i = 0; i < n; ++i)
        if (anchors[i] >= c->n_nodes) return c->fail(EP_ERR_INVALID_ARG, "anchor id out of range");
    if (!n) return EP_OK;
    BatchState h{};
    h.pass = 1;
    h.step = step;
    h.n_anchors = n;
    if (!c->st_inj.ensure(sizeof(BatchState))) return c->fail(EP_ERR_OOM, "state allocation failed");
    BatchState* st = c->st_inj.as<BatchState>();
    cudaStream_t s = c->stream;
    CK(cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s), "inject state");
    CK(cudaMemcpyAsync(c->anchors.p, anchors, (size_t)n * 4, cudaMemcpyHostToDevice, s), "stage anchors");
    launch_sample(sample_params(c, st, false, 2), s);
    CK(cudaGetLastError(), "sample launch");
    std::vector<uint32_t> hn((size_t)n * c->Kcap), hc(n);
    std::vector<float> hw((size_t)n * c->Kcap);
    CK(cudaMemcpyAsync(hc.data(), c->nbr_cnt.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s), "read samples");
    CK(cudaMemcpyAsync(hn.data(), c->nbr.p, hn.size() * 4, cudaMemcpyDeviceToHost, s), "read samples");
    CK(cudaMemcpyAsync(hw.data(), c->nbr_w.p, hw.size() * 4, cudaMemcpyDeviceToHost, s), "read samples");
    CK(cudaMemcpyAsync(neg, c->neg.p, (size_t)n * c->R * 4, cudaMemcpyDeviceToHost, s), "read samples");
    CK(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s), "read state");
    CK(cudaStreamSynchronize(s), "sample");
    if (h.error) return c->fail(EP_ERR_DEVICE, "device error flags 0x%x", h.error);
    for (uint32_t a = 0; a < n; ++a) {
        nbr_cnt[a] = hc[a];
        for (uint32_t k = 0; k < hc[a]; ++k) {
            nbr[(size_t)a * stride + k] = hn[(size_t)a * c->Kcap + k];
            nbr_w[(size_t)a * stride + k] = hw[(size_t)a * c->Kcap + k];
        }
    }
    return EP_OK;
}

extern "C" int ep_get_split(ep_ctx* c, uint32_t* train_ids, uint32_t* valid_ids, uint32_t* n_train,
                            uint32_t* n_valid) {
    if (!c) return EP_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    int rc = prepare_train(c);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream), "split");
    if (train_ids)
        CK(cudaMemcpy(train_ids, c->train_ids.p, (size_t)c->n_train * 4, cudaMemcpyDeviceToHost), "read split");
    if (valid_ids && c->n_valid)
        CK(cudaMemcpy(valid_ids, c->valid_ids.p, (size_t)c->n_valid * 4, cudaMemcpyDeviceToHost), "read split");
    if (n_train) *n_train = c->n_train;
    if (n_valid) *n_valid = c->n_valid;
    return EP_OK;
}

extern "C" int ep_sample_validation(ep_ctx* c, uint32_t first, uint32_t n, uint32_t stride, uint32_t* anchors,
                                    uint32_t* nbr_cnt, uint32_t* nbr, float* nbr_w, uint32_t* neg) {
    if (!c) return EP_ERR_INVALID_ARG;
    if (n && (!anchors || !nbr_cnt || !nbr || !nbr_w || !neg)) return c->fail(EP_ERR_INVALID_ARG, "null array");
    cudaSetDevice(c->device);
    int rc = prepare_train(c);
    if (rc) return rc;
    if (n > c->Bcap) return c->fail(EP_ERR_INVALID_ARG, "%u anchors exceed the batch size %u", n, c->Bcap);
    if ((uint64_t)first + n > c->n_valid)
        return c->fail(EP_ERR_INVALID_ARG, "positions [%u, %llu) beyond the %u validation ids", first,
                       (unsigned long long)first + n, c->n_valid);
    if (stride < c->Kcap)
        return c->fail(EP_ERR_INVALID_ARG, "neighbour stride %u below the %u slots an anchor can fill", stride, c->Kcap);
    if (!n) return EP_OK;
    BatchState h{};
    h.pass = 1;
    h.step = 1;
    h.b0 = first;
    h.n_anchors = n;
    if (!c->st_inj.ensure(sizeof(BatchState))) return c->fail(EP_ERR_OOM, "state allocation failed");
    BatchState* st = c->st_inj.as<BatchState>();
    cudaStream_t s = c->stream;
    CK(cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s), "validation state");
    launch_sample(sample_params(c, st, true, 0), s);   // the validation pass's sampler, as run_validation launches it
    CK(cudaGetLastError(), "sample launch");
    std::vector<uint32_t> hn((size_t)n * c->Kcap), hc(n);
    std::vector<float> hw((size_t)n * c->Kcap);
    CK(cudaMemcpyAsync(anchors, c->anchors.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s), "read samples");
    CK(cudaMemcpyAsync(hc.data(), c->nbr_cnt.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s), "read samples");
    CK(cudaMemcpyAsync(hn.data(), c->nbr.p, hn.size() * 4, cudaMemcpyDeviceToHost, s), "read samples");
    CK(cudaMemcpyAsync(hw.data(), c->nbr_w.p, hw.size() * 4, cudaMemcpyDeviceToHost, s), "read samples");
    CK(cudaMemcpyAsync(neg, c->neg.p, (size_t)n * c->R * 4, cudaMemcpyDeviceToHost, s), "read samples");
    CK(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s), "read state");
    CK(cudaStreamSynchronize(s), "validation samples");
    if (h.error) return c->fail(EP_ERR_DEVICE, "device error flags 0x%x", h.error);
    for (uint32_t a = 0; a < n; ++a) {
        nbr_cnt[a] = hc[a];
        for (uint32_t k = 0; k < hc[a]; ++k) {
            nbr[(size_t)a * stride + k] = hn[(size_t)a * c->Kcap + k];
            nbr_w[(size_t)a * stride + k] = hw[(size_t)a * c->Kcap + k];
        }
    }
    return EP_OK;
}

extern "C" int ep_batch_grad(ep_ctx* c, const ep_batch_samples* sm, ep_sparse_grad* out) {
    if (!c || !out) return EP_ERR_INVALID_ARG;
    if (!c->table_ok) return c->fail(EP_ERR_STATE, "set the table first");
    cudaSetDevice(c->device);
    int rc = stage_samples(c, sm, 4, c->stream);
    if (rc) return rc;
    const uint32_t B = sm->n_anchors;
    rc = run_injected(c, B, c->tt, c->table.p, c->loss.p, nullptr, OUT_DENSE, nullptr, 0.f, 1, c->stream);
    if (rc) return rc;
    uint32_t nt = 0;
    CK(cudaMemcpy(&nt, c->n_touched.p, 4, cudaMemcpyDeviceToHost), "read touched count");
    out->n_rows = nt;
    if (out->loss) CK(cudaMemcpy(out->loss, c->loss.p, (size_t)B * 4, cudaMemcpyDeviceToHost), "read loss");
    if (out->status) CK(cudaMemcpy(out->status, c->status.p, (size_t)B * 4, cudaMemcpyDeviceToHost), "read status");
    if (nt > out->capacity) return c->fail(EP_ERR_INVALID_ARG, "gradient has %u rows, capacity %u", nt, out->capacity);
    if (nt == 0) return EP_OK;
    if (!c->packed.ensure((size_t)nt * c->dims * 4)) return c->fail(EP_ERR_OOM, "pack allocation failed");
    launch_pack_rows(4, c->gdense.p, c->touched.as<uint32_t>(), c->n_touched.as<uint32_t>(), c->dpad, c->dims, c->packed.p,
                     0, nt, c->stream);
    std::vector<uint32_t> ids(nt);
    std::vector<float> rows((size_t)nt * c->dims);
    CK(cudaMemcpyAsync(ids.data(), c->touched.p, (size_t)nt * 4, cudaMemcpyDeviceToHost, c->stream), "read ids");
    CK(cudaMemcpyAsync(rows.data(), c->packed.p, rows.size() * 4, cudaMemcpyDeviceToHost, c->stream), "read rows");
    CK(cudaStreamSynchronize(c->stream), "read gradient");
    // ascending feature order (the device list order depends on scheduling)
    std::vector<uint32_t> ord(nt);
    for (uint32_t i = 0; i < nt; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](uint32_t x, uint32_t y) { return ids[x] < ids[y]; });
    for (uint32_t i = 0; i < nt; ++i) {
        out->feat_ids[i] = ids[ord[i]];
        memcpy(out->rows + (size_t)i * c->dims, rows.data() + (size_t)ord[i] * c->dims, (size_t)c->dims * 4);
    }
    return EP_OK;
}

extern "C" int ep_batch_step(ep_ctx* c, const ep_batch_samples* sm, float lr, uint32_t pass) {
    if (!c) return EP_ERR_INVALID_ARG;
    if (!c->table_ok) return c->fail(EP_ERR_STATE, "set the table first");
    cudaSetDevice(c->device);
    int rc = stage_samples(c, sm, 4, c->stream);
    if (rc) return rc;
    if (c->cfg.form == EP_FORM_PLAIN_FP32)
        return run_injected(c, sm->n_anchors, c->tt, c->table.p, c->loss.p, nullptr, OUT_DENSE, c->table.p, lr, pass, c->stream);
    return run_injected(c, sm->n_anchors, c->tt, c->table.p, c->loss.p, nullptr, OUT_ADAM, c->table.p, lr, pass, c->stream);
}

// autograd: the caller's dense table (n_feat x dims) is copied into the padded
// device layout when dims is not a multiple of the lane width.
static int ag_prepare(ep_ctx* c, const ep_batch_samples* sm, int precision, const void* table_dev, cudaStream_t s) {
    if (!c->graph_ok || !c->feats_ok) return c->fail(EP_ERR_STATE, "upload the graph and the features first");
    if (precision != 0 && precision != 1) return c->fail(EP_ERR_INVALID_ARG, "precision must be 0 or 1");
    const uint32_t es = precision ? 8 : 4;
    int rc = stage_samples(c, sm, es, s);
    if (rc) return rc;
    c->ag_precision = precision;
    c->ag_n = sm->n_anchors;
    if (c->dims == c->dpad && ((uintptr_t)table_dev % 16) == 0) {
        c->ag_table_ptr = table_dev;
    } else {
        if (!c->ag_table.ensure((size_t)c->n_feat * c->dpad * es)) return c->fail(EP_ERR_OOM, "table staging failed");
        CK(cudaMemsetAsync(c->ag_table.p, 0, (size_t)c->n_feat * c->dpad * es, s), "table staging");
        CK(cudaMemcpy2DAsync(c->ag_table.p, (size_t)c->dpad * es, table_dev, (size_t)c->dims * es, (size_t)c->dims * es,
                             c->n_feat, cudaMemcpyDeviceToDevice, s), "table staging");
        c->ag_table_ptr = c->ag_table.p;
    }
    return EP_OK;
}

extern "C" int ep_ag_forward(ep_ctx* c, const ep_batch_samples* sm, int precision, const void* table_dev, void* loss_dev,
                             void* stream) {
    if (!c || !table_dev || !loss_dev) return c ? c->fail(EP_ERR_INVALID_ARG, "null pointer") : EP_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    int rc = ag_prepare(c, sm, precision, table_dev, s);
    if (rc) return rc;
    return run_injected(c, c->ag_n, precision ? TT_F64 : TT_F32, c->ag_table_ptr, loss_dev, nullptr, OUT_DENSE, nullptr, 0.f,
                        1, s);
}

extern "C" int ep_ag_backward(ep_ctx* c, const void* dloss_dev, void* grad_dev, void* stream) {
    if (!c || !dloss_dev || !grad_dev) return c ? c->fail(EP_ERR_INVALID_ARG, "null pointer") : EP_ERR_INVALID_ARG;
    if (c->ag_precision < 0) return c->fail(EP_ERR_STATE, "call ep_ag_forward first");
    cudaSetDevice(c->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    const int tt = c->ag_precision ? TT_F64 : TT_F32;
    const size_t es = c->ag_precision ? 8 : 4;
    int rc = run_injected(c, c->ag_n, tt, c->ag_table_ptr, c->loss.p, dloss_dev, OUT_DENSE, nullptr, 0.f, 1, s);
    if (rc) return rc;
    CK(cudaMemsetAsync(grad_dev, 0, (size_t)c->n_feat * c->dims * es, s), "clear gradient");
    launch_pack_rows(es, c->gdense.p, c->touched.as<uint32_t>(), c->n_touched.as<uint32_t>(), c->dpad, c->dims, grad_dev, 1,
                     (uint32_t)std::min<uint64_t>(c->n_feat, c->items_cap), s);
    CK(cudaGetLastError(), "gradient scatter");
    CK(cudaStreamSynchronize(s), "autograd backward");
    return EP_OK;
}

extern "C" int ep_get_launch_shape(ep_ctx* c, ep_launch_shape* out) {
    if (!c || !out) return EP_ERR_INVALID_ARG;
    out->chunk = c->chunk;
    out->fused_mode = c->fused_mode;
    out->graph_batches = c->graph_batches;
    out->gather_ctas = c->gather_ctas;
    out->ring_reduce_warps = c->ring_pw;
    out->ring_adam_warps = c->ring_cw;
    out->ring_slots = c->ring_slots;
    out->queue_ctas_per_sm = c->queue_ctas;
    out->gather_warps = c->gather_warps;
    out->ring_active = c->cfg.form == EP_FORM_FUSED_BF16 && fused_out_mode(c) == OUT_RING;
    out->tuned = c->tuned;
    out->autotune = c->cfg.autotune;
    return EP_OK;
}

extern "C" int ep_get_tuning(ep_ctx* c, uint32_t* chunk, int32_t* fused_mode, uint32_t* graph_batches) {
    if (!c) return EP_ERR_INVALID_ARG;
    if (chunk) *chunk = c->chunk;
    if (fused_mode) *fused_mode = c->fused_mode;
    if (graph_batches) *graph_batches = c->graph_batches;
    return c->tuned ? EP_OK : 1;
}

// ---------------------------------------------------------------------------
// Table download without device allocation (no counterpart in the reference).
//
// ep_get_table stages the whole table as dense FP32 in a context buffer that
// it allocates on first use: n_feat * dims * 4 bytes, 10 GB for 10M features
// at 256 dims.  Some callers cannot allocate device memory at that point: a
// process whose HBM is already held by the table and by a caching allocator
// or memory pool, or a serving loop that reads rows while other work runs and
// must not call cudaMalloc/cudaFree (which can synchronise the device).
// ep_get_table_static reads a window of rows through a fixed scratch that is
// part of the library's static device image, so the call allocates nothing.
//
// The scratch belongs to the device, not to a context: calls on one device
// that overlap in time (from two host threads, or two contexts on different
// streams) write the same scratch and corrupt each other's rows, so callers
// serialise them.  Nothing in the scratch has to start at zero: each call
// writes every element it copies out before the copy.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kStaticScratchBytes = (size_t)8 << 20;   // 8 MiB
static_assert(kStaticScratchBytes == (size_t)EP_STATIC_SCRATCH_BYTES, "header and scratch size disagree");
constexpr int kStaticMaxDevices = 64;

__device__ __align__(256) float g_static_scratch[kStaticScratchBytes / sizeof(float)];

std::mutex g_static_mu;
float* g_static_ptr[kStaticMaxDevices] = {};   // device address of g_static_scratch, per device

// Looks up the scratch's device address once per device; the device must be
// current.  Only the address returned here is handed to kernels and copies.
cudaError_t static_scratch(int device, float** out) {
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_ptr[device]) {
        float* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_static_scratch);
        if (e != cudaSuccess) return e;
        g_static_ptr[device] = p;
    }
    *out = g_static_ptr[device];
    return cudaSuccess;
}

}  // namespace

extern "C" int ep_get_table_static(ep_ctx* c, uint64_t first_row, uint64_t n_rows, float* out) {
    if (!c) return EP_ERR_INVALID_ARG;
    if (!out && n_rows) return c->fail(EP_ERR_INVALID_ARG, "out is NULL");
    if (!c->table_ok) return c->fail(EP_ERR_STATE, "no table");
    if (first_row > c->n_feat || n_rows > c->n_feat - first_row)
        return c->fail(EP_ERR_INVALID_ARG, "rows [%llu, %llu) outside the table's %u rows",
                       (unsigned long long)first_row, (unsigned long long)(first_row + n_rows), c->n_feat);
    const uint64_t row_bytes = (uint64_t)c->dims * sizeof(float);
    const uint64_t max_rows = kStaticScratchBytes / row_bytes;
    if (n_rows > max_rows)
        return c->fail(EP_ERR_INVALID_ARG,
                       "%llu rows exceed the %zu-byte static scratch: at most %llu rows of %u dims per call",
                       (unsigned long long)n_rows, kStaticScratchBytes, (unsigned long long)max_rows, c->dims);
    if (c->device < 0 || c->device >= kStaticMaxDevices)
        return c->fail(EP_ERR_UNSUPPORTED, "device %d beyond the %d devices the static scratch serves", c->device,
                       kStaticMaxDevices);
    CK(cudaSetDevice(c->device), "select device");
    float* scratch = nullptr;
    CK(static_scratch(c->device, &scratch), "cudaGetSymbolAddress of the static scratch");
    if (!n_rows) return EP_OK;
    const size_t es = c->tt == TT_BF16 ? 2 : (c->tt == TT_F32 ? 4 : 8);
    const char* rows = c->table.as<const char>() + first_row * c->dpad * es;
    launch_convert_table(c->tt, const_cast<char*>(rows), scratch, n_rows, c->dims, c->dpad, 0, c->stream);
    CK(cudaGetLastError(), "static table download");
    CK(cudaMemcpyAsync(out, scratch, n_rows * row_bytes, cudaMemcpyDeviceToHost, c->stream), "static table download");
    CK(cudaStreamSynchronize(c->stream), "static table download");
    return EP_OK;
}
