// ep_internal.h -- structures shared by the host driver (ep_ctx.cu) and the
// kernel translation units (ep_fwd.cu, ep_sort.cu, ep_red.cu).
//
// Per-batch data flow on the device (stream launches in this order; replayed
// graphs run the scan, item emission and sort on a side stream beside the
// gathers and the loss, and the fix-ups beside the next batch's sampling):
//   k_batch_begin  -> BatchState (batch range, lr, Adam bias corrections)
//   k_sample       -> anchors, sampled neighbours, negatives, occurrence counts
//   k_scan_occ     -> exclusive item offsets per anchor
//   k_forward      -> role means, loss, per-role gradient directions and
//                     scales, one item (feature, role-src, count) per feature
//                     occurrence, written at deterministic offsets
//   radix sort     -> items stably ordered by feature id
//   k_reduce       -> per-feature gradient = sum over kept items, with the
//                     first-occurrence rule; fused Adam (FUSED) or a dense
//                     gradient row + touched list (PLAIN / parity hooks);
//                     queues the spans longer than FIX_SHORT later chunks
//   k_fixup        -> features whose items span up to FIX_SHORT later chunks
//   k_fixup_long   -> the longer spans (independent of k_fixup)
//   k_adam         -> (PLAIN) Adam over the touched list
//   k_batch_end    -> deterministic loss sums, counters, state advance
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ep {

// Device error bits (BatchState::error).  A kernel that detects a condition
// it cannot handle sets a bit and skips the offending work; the host reads
// the word after each pass / synchronisation and reports EP_ERR_DEVICE.
enum : uint32_t {
    ERR_ITEMS_OVERFLOW = 1u << 0,   // a batch emitted more items than allocated
    ERR_FEISTEL = 1u << 1,          // permutation cycle walk exceeded its cap
    ERR_NBR_OVERFLOW = 1u << 2,     // sampled neighbours exceeded capacity
    ERR_RING_TIMEOUT = 1u << 3,     // a wait of the reducer's row ring gave up (bounded polls)
};

// OUT_ADAM: each finished feature row is updated in place by the warp that
// finished it.  OUT_DENSE: rows go to a dense gradient buffer plus a touched
// list (a separate Adam kernel, or the caller, consumes them).  OUT_QUEUE:
// rows are queued in the warp's shared memory, their Adam state copied in
// asynchronously, and the oldest updated when the queue is full.
// OUT_RING: warp-specialised CTAs; reducing warps push finished rows into a
// CTA-wide shared-memory ring whose slots bulk-copy (TMA) the row's Adam
// state, and Adam warps pop and update them.
enum OutMode : int { OUT_ADAM = 0, OUT_DENSE = 1, OUT_QUEUE = 2, OUT_RING = 3 };
enum TableType : int { TT_F32 = 0, TT_BF16 = 1, TT_F64 = 2 };

struct BatchState {
    uint32_t pass;          // 1-based pass index
    uint32_t batch;         // batch index within the pass
    uint64_t step;          // global optimizer step, starts at 1 (mod.rs:153)
    uint32_t step_cur;      // low bits of the step of the batch in flight (set by k_batch_begin), read
                            // by the Adam kernels while k_batch_end may already advance `step`
    uint32_t b0;            // first position of this batch in the pass order
    uint32_t n_anchors;     // anchors in this batch
    float lr;               // cos-decay learning rate for `step`
    float bc1, bc2;         // 1 - beta^t with t = pass + 1 (optimizer.rs:50)
    uint32_t error;         // ERR_* bits, sticky
    uint32_t n_items;       // items emitted by this batch
    uint32_t fwd_next;      // work queue of the persistent gather: next anchor to take (k_batch_begin zeroes it)
    uint32_t red_next;      // work queue of the persistent reducer: next chunk to take (k_batch_begin zeroes it)
    float noise_sigma;      // gradient-noise scale of this step (0 = off)
    // per-batch outputs of k_batch_end
    float batch_err;        // sum(loss kept) / n_anchors (0 when none kept)
    uint32_t batch_kept;
    // pass accumulators (reset by the host at a pass start)
    double pass_err_sum;
    uint32_t pass_batches;
    uint32_t n_long[2];     // long spans queued by k_reduce for k_fixup_long, by the step's parity: a
                            // batch's k_batch_begin zeroes its own while the previous batch's
                            // k_fixup_long may still read the other
    // the batch's item count and Adam constants as k_reduce found them: the
    // fix-up and dense Adam kernels read these, so that in replayed graphs
    // the next batch's k_batch_begin and sampler may run beside them
    uint32_t fx_items, fx_step;
    float fx_lr, fx_bc1, fx_bc2, fx_sigma;
    unsigned long long anchors, kept, nan_anchors, items, gathered, unique_rows, sampled;
    double valid_sum;
};

// Feature dropout (max_features): EP_SAMPLE_* kind, Fixed count k,
// Probability p and its key threshold p * 2^32, and the Philox key.
struct FeatDrop {
    int kind;
    uint32_t k;
    float p;
    uint32_t thr;
    uint64_t seed;
};

struct SampleCfg {
    int nodes_kind;         // EP_SAMPLE_*
    float nodes_val;
    uint32_t K;             // Fixed(k)
    uint32_t Kcap;          // neighbour slots per anchor
    uint32_t R;             // negatives
    int weighted_avg;       // weighted_neighbor_averaging
    int weighted_sampling;  // weighted_neighbor_sampling (with weighted averaging: A-Res)
    FeatDrop fd;            // feature dropout of every role node
    uint32_t hard;          // hard negatives from random walks (0 = off)
    int ppr;                // PPR loss: positives are R random-walk end nodes
    float ppr_restart;      // its restart probability
    uint64_t seed;
};

struct SampleParams {
    BatchState* st;
    SampleCfg cfg;
    const uint64_t* row_ptr;
    const uint32_t* cols;
    const float* wcdf;
    const uint64_t* fptr;
    const uint32_t* order;  // anchor source (train or valid ids)
    uint32_t n_order;
    const uint32_t* pool;   // negative pool (train or valid ids)
    uint32_t n_pool;
    uint32_t batch_cap;     // anchors per batch
    uint32_t sample_warps;  // warps per CTA (1-8; 0 = 8)
    int injected;           // 1: samples provided by the host (only count);
                            // 2: anchors provided, neighbours and negatives sampled
    int eval;               // validation: fixed sampling stream, no shuffle
    uint32_t feistel_half;  // half-width in bits of the permutation domain
    uint32_t feistel_key[4];
    // outputs
    uint32_t* anchors;
    uint32_t* nbr;
    float* nbr_w;
    uint32_t* nbr_cnt;
    uint32_t* neg;
    uint32_t* occ;          // per-anchor item counts
};

struct ForwardParams {
    BatchState* st;
    int loss;               // EP_LOSS_*
    float gamma, neg_margin;
    int loss_weighting;
    float lw_exp;
    FeatDrop fd;            // feature dropout (same keys as the sampler's counts)
    int eval;               // validation batch (fixed sampling salt)
    uint32_t R, Kcap, dims, dpad;
    const uint64_t* row_ptr;
    const uint64_t* fptr;
    const uint32_t* fids;
    const void* table;      // T[n_feat * dpad]
    const uint32_t* anchors;
    const uint32_t* nbr;
    const float* nbr_w;
    const uint32_t* nbr_cnt;
    const uint32_t* neg;
    const uint32_t* occ_off;  // exclusive offsets, [n_anchors] = total
    const float* dloss;       // optional per-anchor upstream gradient (autograd)
    int dloss_f64;
    int emit;                 // 0: forward only (validation)
    uint64_t items_cap;
    uint8_t* deferred;        // [n_anchors]: 1 = anchor left to the direct path
    uint32_t gather_warps;    // warps per CTA of the one-warp-per-anchor gather and item emission (1-8; 0 = 8)
    uint32_t gather_ctas;     // staged gather: 0 = a warp per anchor; else this many persistent CTAs
                              // whose warps take anchors from BatchState::fwd_next
    // outputs
    void* dir;              // A[n_anchors * NR * dpad]: role means, then (D == A) directions
    void* dir16;            // BF16 tables: directions as BF16 (D = bf16)
    void* scale;            // A[n_anchors * NR]
    uint8_t* valid;         // [n_anchors * NR]
    void* loss_out;         // A[n_anchors]
    int means_dead;         // k_fwd_loss drops the role means from L2 once read (no reader after it)
    int32_t* status;        // [n_anchors]
    uint32_t* item_f;
    uint32_t* item_src;
    float* item_c;
};

struct ReduceParams {
    BatchState* st;
    uint32_t NR, dpad, chunk;
    int grad_true;          // EP_GRAD_TRUE
    int out_mode;           // OutMode
    const uint32_t* skey;   // sorted feature ids
    const uint2* sval;      // (role-src, count-weight bits) of each sorted item
    const void* dir;        // directions when D == A
    const void* dir16;      // directions when D == bf16 (BF16 tables)
    const void* scale;      // A
    const uint8_t* valid;
    // OUT_ADAM
    void* table;            // T
    float* m;
    float* v;
    uint64_t seed;
    // OUT_DENSE
    void* gdense;           // A[n_feat * dpad]
    uint32_t* touched;      // list of touched features
    uint32_t* n_touched;
    // carries
    void* carry_head;       // A[n_chunks * dpad]
    void* carry_tail;
    uint32_t* carry_f;
    uint32_t* carry_flags;
    uint32_t* long_list;    // owner chunks of long spans [2][long_cap], by step parity
    uint32_t long_cap;
    // OUT_RING shape: reducing warps, Adam warps and ring slots per CTA
    uint32_t ring_pw, ring_cw, ring_slots;
    // OUT_QUEUE: resident CTAs per SM the reducer is compiled for (4 or 5)
    uint32_t queue_ctas_per_sm;
    // 0: one warp per chunk (static stride); else a persistent grid of this
    // many CTAs whose warps take chunks from BatchState::red_next
    uint32_t red_ctas;
};

// ---- launchers (defined in the kernel translation units) -----------------
void launch_batch_begin(BatchState* st, uint32_t n_order, uint32_t batch_cap,
                        uint32_t steps_per_pass, uint64_t total_steps, uint64_t warmup,
                        float alpha, int injected, float noise, float noise_decay, cudaStream_t s);
void launch_sample(const SampleParams& p, cudaStream_t s);
void launch_scan_occ(BatchState* st, uint32_t* occ, uint32_t cap, uint64_t items_cap,
                     cudaStream_t s);
// part: FWD_ALL, the gathers alone (they emit the items when ForwardParams
// says so), the loss alone, or the item emission alone (k_fwd_emit)
enum ForwardPart : int { FWD_ALL = 0, FWD_GATHER = 1, FWD_LOSS = 2, FWD_EMIT = 3 };
void launch_forward(int tt, int vpl, const ForwardParams& p, uint32_t cap, cudaStream_t s, int part = FWD_ALL);
void launch_radix_sort(BatchState* st, uint32_t* keys, uint32_t* keys_alt, const uint32_t* item_src,
                       const float* item_c, uint2* vals, uint2* vals_alt, uint32_t* hist, uint64_t cap,
                       int key_bits, uint32_t** sorted_keys, uint2** sorted_vals, cudaStream_t s);
void launch_reduce(int tt, int vpl, const ReduceParams& p, uint64_t items_cap, cudaStream_t s);
// part: 0 both fix-up kernels in order, 1 the short spans (k_fixup), 2 the
// long spans (k_fixup_long); the two parts are independent
void launch_fixup(int tt, int vpl, const ReduceParams& p, uint64_t items_cap, cudaStream_t s, int part = 0);
void launch_adam_dense(int tt, int vpl, BatchState* st, void* table, float* m, float* v,
                       const float* g, const uint32_t* touched, const uint32_t* n_touched,
                       uint32_t dpad, uint32_t max_rows, uint64_t seed, cudaStream_t s);
void launch_batch_end(BatchState* st, const void* loss, const int32_t* status,
                      const uint32_t* nbr_cnt, uint32_t cap, uint32_t steps_per_pass,
                      int eval, int loss_f64, cudaStream_t s);
void launch_init_table(int tt, void* table, uint64_t n_feat, uint32_t dims, uint32_t dpad,
                       uint64_t seed, cudaStream_t s);
// Writes the table as dense FP32 [n_feat x dims] to out_dev (device memory,
// or page-locked host memory through its device address); false when the
// shape or alignment needs the element-wise conversion instead.
bool launch_table_out(int tt, const void* table, float* out_dev, uint64_t n_feat, uint32_t dims, uint32_t dpad,
                      cudaStream_t s);
void launch_convert_table(int tt_dst, void* dst, const float* src, uint64_t n_feat,
                          uint32_t dims, uint32_t dpad, int to_device_layout, cudaStream_t s);
void launch_node_bound(const uint64_t* row_ptr, const uint32_t* cols, const uint64_t* fptr, uint32_t n,
                       int nodes_kind, uint32_t K, uint32_t R, uint32_t max_feat, int ppr, uint32_t* bound,
                       cudaStream_t s);
void launch_split(uint32_t* train, uint32_t n_train, uint32_t* valid, uint32_t n, uint64_t seed,
                  uint32_t half, uint32_t* err, cudaStream_t s);
void launch_pack_rows(size_t es, const void* dense, const uint32_t* rows, const uint32_t* n_rows,
                      uint32_t dpad, uint32_t dims, void* out, int scatter, uint32_t max_rows,
                      cudaStream_t s);
size_t radix_hist_entries(uint64_t cap);
uint32_t reduce_chunks(uint64_t cap, uint32_t chunk);
cudaError_t reduce_kernels_setup();
// Whether OUT_RING serves this row shape (whole rows of m, v and the table are
// 16-byte multiples, and the ring's shared memory fits), and the ring's
// shared memory per CTA.
bool ring_supported(int tt, uint32_t dpad, uint32_t pw, uint32_t cw, uint32_t slots);
size_t ring_smem_bytes(int tt, uint32_t dpad, uint32_t pw, uint32_t slots);

}  // namespace ep
