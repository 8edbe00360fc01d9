/*
 * ep_gb300.h -- C ABI of the GB300 (sm_103a) Embedding Propagation trainer.
 *
 * This is the boundary a host binding (the reference's PyO3 module, a Rust
 * extern "C" crate, or the ctypes layer in cloverleaf_gb300/) calls in place
 * of cloverleaf's CPU training path:
 *
 *   EmbeddingPropagator.__new__        src/lib.rs:1205-1307  -> ep_config + ep_create
 *   EmbeddingPropagator.learn_features src/lib.rs:1327-1370  -> ep_upload_graph,
 *        ep_upload_features, ep_set_table, ep_train, ep_get_table
 *   EmbeddingPropagation::learn        src/algos/ep/mod.rs:80-287 -> ep_train
 *
 * Conventions: every function returns an ep_status (0 = EP_OK, negative =
 * error) except ep_last_error/ep_destroy/ep_config_default.  No exception or
 * signal crosses the ABI.  The caller owns every host buffer; the context owns
 * all device memory.  One context per host thread; each context owns one CUDA
 * stream.  Node ids are u32 (< 2^32 nodes), CSR row pointers are u64.
 */
#ifndef EP_GB300_H
#define EP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EP_ABI_VERSION 2u

typedef struct ep_ctx ep_ctx;

typedef enum ep_status {
    EP_OK = 0,
    EP_ERR_INVALID_ARG = -1,   /* bad pointer, size or config value */
    EP_ERR_CUDA = -2,          /* a CUDA runtime call failed */
    EP_ERR_OOM = -3,           /* device allocation failed */
    EP_ERR_STATE = -4,         /* call out of order (e.g. train before upload) */
    EP_ERR_DEVICE = -5,        /* a kernel raised its device error flag */
    EP_ERR_UNSUPPORTED = -6,   /* option not implemented on this path */
    EP_ERR_NO_DEVICE = -7      /* no usable CUDA device */
} ep_status;

/* Loss (src/algos/ep/loss.rs:15-38, constructors src/lib.rs:988-1103).
 * RANK and RANKSPACE take tau in `gamma`; PPR is the margin loss with
 * random-walk positives (`negatives` walks, restart `ppr_restart_p`). */
enum {
    EP_LOSS_MARGIN = 0,
    EP_LOSS_STARSPACE = 1,
    EP_LOSS_CONTRASTIVE = 2,
    EP_LOSS_RANK = 3,
    EP_LOSS_RANKSPACE = 4,
    EP_LOSS_PPR = 5
};
/* Sample kind for max_nodes / max_features (src/algos/utils.rs:165-184). */
enum { EP_SAMPLE_ALL = 0, EP_SAMPLE_FIXED = 1, EP_SAMPLE_PROB = 2 };
/* Loss weighting (src/algos/ep/mod.rs:31-36, src/lib.rs:941-960). */
enum { EP_LW_NONE = 0, EP_LW_LOG = 1, EP_LW_EXP = 2 };
/* Implementation form.  PLAIN_FP32: FP32 table, one kernel per stage, the
 * batch gradient materialised before a separate Adam kernel.  FUSED_BF16:
 * BF16 table (stochastic rounding) with FP32 accumulation and FP32 Adam
 * moments, gradient reduction fused with Adam, replayed as a CUDA graph. */
enum { EP_FORM_PLAIN_FP32 = 0, EP_FORM_FUSED_BF16 = 1 };
/* Gradient extraction.  REFERENCE: a feature's per-anchor gradient comes from
 * the first role (h(v), ~h(v), h(u_1..R)) in which it has a finite gradient
 * (src/algos/ep/mod.rs:361-378).  TRUE: all roles' contributions are summed
 * (the derivative of the loss). */
enum { EP_GRAD_REFERENCE = 0, EP_GRAD_TRUE = 1 };

typedef struct ep_config {
    uint32_t abi_version;        /* must be EP_ABI_VERSION */
    float alpha;                 /* peak learning rate (lib.rs:1263, default 0.9) */
    int32_t loss;                /* EP_LOSS_* (default margin) */
    float gamma;                 /* margin / positive margin / tau (default 1) */
    float neg_margin;            /* contrastive negative margin */
    uint32_t negatives;          /* negatives per anchor (default 1) */
    uint32_t batch_size;         /* default 50 */
    uint32_t dims;               /* default 100 */
    uint32_t passes;             /* default 100 */
    uint64_t seed;               /* default 20222022 (lib.rs:90) */
    int32_t max_nodes_kind;      /* EP_SAMPLE_*, reconstruction neighbours */
    float max_nodes;             /* Fixed: count, Prob: p */
    int32_t max_features_kind;   /* EP_SAMPLE_* */
    float max_features;
    int32_t weighted_neighbor_sampling;
    int32_t weighted_neighbor_averaging;
    int32_t loss_weighting;      /* EP_LW_* */
    float loss_weighting_exp;
    float valid_pct;             /* default 0.1 */
    uint32_t hard_negatives;     /* default 0 */
    float noise;                 /* gradient noise, default 0 */
    int32_t form;                /* EP_FORM_* */
    int32_t grad_mode;           /* EP_GRAD_* */
    int32_t device;              /* CUDA device ordinal */
    int32_t use_graphs;          /* replay each batch as a CUDA graph */
    int32_t autotune;            /* pick launch shapes by timing candidates on the
                                    first training batches (see ep_get_launch_shape):
                                    0 off; 1 (default) only shapes that leave results
                                    bit-identical; 2 also reducer chunk sizes, whose
                                    summation order then depends on timing.  Setting a
                                    shape through EP_FUSED_MODE, EP_REDUCE_CHUNK,
                                    EP_GATHER_CTAS or EP_RING_* in the environment
                                    turns tuning off */
    float ppr_restart_p;         /* EP_LOSS_PPR walk restart probability in [0, 1] */
} ep_config;

typedef struct ep_pass_stats {
    uint32_t pass;               /* 1-based */
    uint32_t batches;
    float train_loss;            /* mean over batches of sum(loss)/batch_len (mod.rs:256-265) */
    float valid_loss;            /* NaN when valid_pct == 0 (mod.rs:267-283) */
    float lr_last;
    float noise_last;            /* gradient-noise scale of the last step (0 = off) */
    uint64_t anchors;            /* anchors processed */
    uint64_t kept_anchors;       /* finite loss > 0 */
    uint64_t nan_anchors;
    uint64_t items;              /* emitted (feature, role) gradient items */
    uint64_t gathered_rows;      /* G: distinct (role, feature) rows gathered */
    uint64_t unique_rows;        /* U: rows updated by Adam */
    uint64_t sampled_neighbors;  /* S */
    double ms;                   /* device time of the pass's batches */
    double alg_bytes;            /* G*d*s + U*d*(2s+16) + 4G + 4S + 8*B*(R+2) */
    uint64_t launches;           /* kernels launched for these batches */
} ep_pass_stats;

/* Stages timed by ep_profile_batches. */
enum { EP_STAGE_SAMPLE = 0,      /* batch set-up, sampling, item offsets */
       EP_STAGE_FORWARD = 1,     /* gather-mean, loss, gradient directions, items */
       EP_STAGE_SORT = 2,        /* radix sort of items by feature id */
       EP_STAGE_REDUCE = 3,      /* per-feature reduction (+ fused Adam) and carries */
       EP_STAGE_FIXUP = 4,       /* features spanning reducer chunks */
       EP_STAGE_ADAM = 5,        /* separate Adam kernel (PLAIN form only) */
       EP_STAGE_END = 6,         /* loss sums, counters, state advance */
       EP_N_STAGES = 7 };

/* Explicit samples for the parity hooks (host pointers).  Anchor a has
 * neighbours nbr[nbr_ptr[a] .. nbr_ptr[a+1]) with base weights nbr_w and
 * negatives negatives[a*R .. a*R+R), R = config.negatives. */
typedef struct ep_batch_samples {
    uint32_t n_anchors;
    const uint32_t* anchors;
    const uint32_t* nbr_ptr;     /* n_anchors + 1 */
    const uint32_t* nbr;
    const float* nbr_w;
    const uint32_t* negatives;   /* n_anchors * R */
} ep_batch_samples;

/* Sparse batch gradient returned by ep_batch_grad (host pointers). */
typedef struct ep_sparse_grad {
    uint32_t capacity;           /* rows the caller allocated */
    uint32_t n_rows;             /* out: touched feature rows */
    uint32_t* feat_ids;          /* out: capacity entries, ascending */
    float* rows;                 /* out: capacity * dims */
    float* loss;                 /* out: n_anchors, after loss weighting */
    int32_t* status;             /* out: n_anchors: 0 kept, 1 loss <= 0, 2 NaN */
} ep_sparse_grad;

/* Fills the reference defaults of EmbeddingPropagator.__new__
 * (src/lib.rs:1262-1274) plus form = PLAIN_FP32, grad_mode = REFERENCE. */
void ep_config_default(ep_config* cfg);

/* Validates cfg, selects the device, creates the stream.
 * Replaces EmbeddingPropagator::new (src/lib.rs:1205-1307). */
int ep_create(const ep_config* cfg, ep_ctx** out);

/* Uploads the graph once: CSR row pointers (n_nodes+1), u32 column ids and
 * per-row CDF weights as produced by CumCSR::convert (src/graph.rs:399-422).
 * w_cdf may be NULL (uniform weights).  Rejects non-monotone rows and ids
 * >= n_nodes.  Replaces the borrow of Graph.graph at src/lib.rs:1345. */
int ep_upload_graph(ep_ctx* ctx, uint64_t n_nodes, const uint64_t* row_ptr,
                    const uint32_t* cols, const float* w_cdf);

/* Uploads the node -> feature CSR (FeatureStore, src/feature_store.rs:19-25
 * flattened): fptr (n_nodes+1), fids < n_feat.  Replaces &features.features
 * at src/lib.rs:1347. */
int ep_upload_features(ep_ctx* ctx, uint64_t n_nodes, const uint64_t* fptr,
                       const uint32_t* fids, uint32_t n_feat);

/* Sets the feature table: init (n_feat*dims FP32, row-major) or NULL for the
 * reference's seeded init, rows U(-1,1)^d L2-normalised
 * (src/algos/ep/mod.rs:100-110, 381-392).  Resets the Adam moments and the
 * step counter (a warm start re-initialises them too, mod.rs:114-116). */
int ep_set_table(ep_ctx* ctx, const float* init);

/* Runs config.passes passes (src/algos/ep/mod.rs:156-284).  stats may be NULL;
 * otherwise up to stats_len per-pass records are written. */
int ep_train(ep_ctx* ctx, ep_pass_stats* stats, uint32_t stats_len);

/* Runs n_batches more batches of the pass sequence (the per-batch step of
 * mod.rs:174-261), crossing pass boundaries as ep_train would.  Accumulated
 * counters of the batches run are written to *stats when non-NULL. */
int ep_train_batches(ep_ctx* ctx, uint32_t n_batches, ep_pass_stats* stats);

/* Measurement hook (no counterpart in the reference): runs n_batches more
 * batches like ep_train_batches, but launched stage by stage with CUDA events
 * between the stages, and writes the mean device time per batch of each stage
 * to stage_ms[EP_N_STAGES].  Counters go to *stats when non-NULL. */
int ep_profile_batches(ep_ctx* ctx, uint32_t n_batches, double* stage_ms, ep_pass_stats* stats);

/* Parity hook: loss and reduced batch gradient for explicit samples from the
 * current table, without updating it (mod.rs:183-233 for one batch). */
int ep_batch_grad(ep_ctx* ctx, const ep_batch_samples* samples, ep_sparse_grad* out);

/* Inspection hook (no counterpart in the reference): runs the device sampler
 * for n given anchors (n <= batch_size) at optimizer step `step` (the
 * sampler's random streams are keyed by anchor and step): anchor a's sampled
 * neighbours go to nbr[a*stride .. a*stride + nbr_cnt[a]) with their weights
 * in nbr_w, its negatives (hard ones first, then uniform) to
 * neg[a*R .. a*R + R).  stride must be at least the neighbours an anchor can
 * take (min(max_nodes, max degree) for Fixed, the max degree otherwise). */
int ep_sample(ep_ctx* ctx, const uint32_t* anchors, uint32_t n, uint32_t step, uint32_t stride,
              uint32_t* nbr_cnt, uint32_t* nbr, float* nbr_w, uint32_t* neg);

/* Inspection hook: the train/validation split of mod.rs:119-125 (a seeded
 * permutation; the last floor(n * valid_pct) ids are validation ids).  Writes
 * the n_train training ids (the pool uniform negatives are drawn from,
 * node_sampler.rs:83-107) and the n_valid validation ids in their validation
 * order; either pointer may be NULL.  *n_train / *n_valid receive the counts. */
int ep_get_split(ep_ctx* ctx, uint32_t* train_ids, uint32_t* valid_ids, uint32_t* n_train, uint32_t* n_valid);

/* Inspection hook: the samples the validation pass (mod.rs:267-283) draws for
 * its anchors at positions [first, first + n) of the validation order
 * (n <= batch_size): the anchors, their neighbours (stride as ep_sample) and
 * their negatives, drawn from the validation ids.  Validation sampling uses
 * one fixed random stream, so these are the samples of every pass. */
int ep_sample_validation(ep_ctx* ctx, uint32_t first, uint32_t n, uint32_t stride, uint32_t* anchors,
                         uint32_t* nbr_cnt, uint32_t* nbr, float* nbr_w, uint32_t* neg);

/* Parity hook: one full optimizer step for explicit samples with learning
 * rate lr and Adam time pass+1 (optimizer.rs:43-81). */
int ep_batch_step(ep_ctx* ctx, const ep_batch_samples* samples, float lr, uint32_t pass);

/* Copies the table out as n_feat*dims FP32.  Replaces the EmbeddingStore
 * returned by learn (src/lib.rs:1362-1368).  When out is page-locked host
 * memory (cudaHostAlloc / cudaHostRegister, e.g. a pinned torch tensor) and
 * dims is a multiple of 4, a kernel writes the rows into it directly at the
 * host link's rate; otherwise the rows go through a device staging buffer
 * allocated on first use and one copy. */
int ep_get_table(ep_ctx* ctx, float* out);

/* Launch shapes in use (no counterpart in the reference): the reducer's items
 * per warp, the FUSED form's Adam placement (2 = queued in the reducer, 1 = a
 * separate kernel, 0 = per row as each feature closes, 3 = the
 * warp-specialised ring) and the batches per replayed CUDA graph.  With
 * config.autotune the first training call that asks for enough batches times
 * the candidates on real batches and keeps the fastest; returns EP_OK once
 * that choice is made, 1 before (the values are then the defaults).  Any
 * pointer may be NULL. */
int ep_get_tuning(ep_ctx* ctx, uint32_t* chunk, int32_t* fused_mode, uint32_t* graph_batches);

/* Every launch shape in use (no counterpart in the reference), including
 * those ep_get_tuning does not report: the staged gather's grid (0 = one
 * warp per anchor, else persistent CTAs taking anchors from a work queue)
 * and the ring's reducing warps, Adam warps and slots per CTA. */
typedef struct ep_launch_shape {
    uint32_t chunk;
    int32_t fused_mode;
    uint32_t graph_batches;
    uint32_t gather_ctas;
    uint32_t ring_reduce_warps, ring_adam_warps, ring_slots;
    int32_t ring_active;         /* the FUSED form reduces through the ring */
    uint32_t queue_ctas_per_sm;  /* the queue reducer's resident CTAs per SM (4 or 5) */
    uint32_t gather_warps;       /* warps per CTA of the one-warp-per-anchor gather */
    int32_t tuned;               /* the autotuner has made its choice */
    int32_t autotune;            /* the tuning level in effect */
} ep_launch_shape;
int ep_get_launch_shape(ep_ctx* ctx, ep_launch_shape* out);

/* Row download without device allocation (no counterpart in the reference).
 * Writes rows [first_row, first_row + n_rows) of the table to out (host
 * memory, n_rows * dims FP32), the same values ep_get_table gives for them.
 * ep_get_table stages the whole table in a device buffer it allocates on
 * first use (n_feat * dims * 4 bytes); this call instead goes through a fixed
 * scratch of EP_STATIC_SCRATCH_BYTES in the library's static device image and
 * allocates no device memory.  It is meant for callers that cannot allocate
 * at that point: HBM already held by the table and a memory pool, or a
 * serving loop that must not call cudaMalloc/cudaFree while other work runs.
 * Limit: at most EP_STATIC_SCRATCH_BYTES / (4 * dims) rows per call (4096 rows
 * at 512 dims); a larger window fails with EP_ERR_INVALID_ARG and no work is
 * done.  The first call on each device looks up the scratch's device address;
 * make that first call before any stream capture begins.  The scratch is
 * shared by every context on a device, so calls on one device must not
 * overlap in time (they would overwrite each other's rows).  Nothing in the
 * scratch needs to start at zero. */
#define EP_STATIC_SCRATCH_BYTES (8u << 20)
int ep_get_table_static(ep_ctx* ctx, uint64_t first_row, uint64_t n_rows, float* out);

/* Device-pointer entry points behind the torch.autograd.Function binding.
 * precision: 0 = FP32 table/compute, 1 = FP64 (gradient checks only).
 * ep_ag_forward computes per-anchor losses (loss_dev, n_anchors values of the
 * precision) for explicit samples against table_dev (n_feat*dims);
 * ep_ag_backward consumes dloss_dev (n_anchors values) and writes the dense
 * gradient dL/dtable into grad_dev (n_feat*dims, overwritten).  Both run on
 * `stream` (a cudaStream_t, NULL = the context stream). */
int ep_ag_forward(ep_ctx* ctx, const ep_batch_samples* samples, int precision,
                  const void* table_dev, void* loss_dev, void* stream);
int ep_ag_backward(ep_ctx* ctx, const void* dloss_dev, void* grad_dev, void* stream);

/* Self-check (no counterpart in the reference): rounds n element pairs
 * (hashed from seed, with special values among them) to BF16 both with the
 * hardware stochastic-rounding conversion the FUSED form's Adam uses and with
 * the bit rule it stands for (add 16 random bits below the BF16 mantissa,
 * truncate; NaN and infinities kept), and stores the number of pairs whose
 * results differ in *mismatches (0 expected). */
int ep_selftest_stochastic_rounding(int device, uint64_t n, uint64_t seed, uint64_t* mismatches);

/* Blocks until the context's work is done; reports device error flags. */
int ep_synchronize(ep_ctx* ctx);

/* Message of the last failing call on ctx (or of the last ep_create failure
 * when ctx is NULL).  Valid until the next call on the same context. */
const char* ep_last_error(const ep_ctx* ctx);

void ep_destroy(ep_ctx* ctx);

/* ---- evaluation: node embeddings and nearest neighbours ---------------- */

/* NodeEmbedder.embed_feature_set (src/lib.rs:2092-2124) with AvgAggregator
 * (fweight NULL) or WeightedAggregator (fweight[f] = alpha / (alpha + p_f)),
 * src/algos/aggregator.rs:17-120: out[v] (n_nodes x dims FP32) = the
 * weighted mean of the table rows of v's features fids[fptr[v]..fptr[v+1])
 * in f32 as the reference sums them; featureless nodes get zeros.  Host
 * buffers; dims <= 512.  Errors: ep_knn_last_error(). */
int ep_embed_features(int device, uint64_t n_nodes, const uint64_t* fptr, const uint32_t* fids,
                      const float* fweight, uint32_t n_feat, uint32_t dims, const float* table, float* out);

/* Exact cosine top-k of every query row against every database row
 * (NodeEmbeddings.nearest_neighbor with EDist::Cosine, src/embeddings.rs:
 * 149-173, for n_q queries at once).  Rows are normalised and rounded to
 * BF16; similarities accumulate in FP32 on the tensor cores.  idx_out /
 * sim_out (n_q x k) get the k most similar database rows per query in
 * decreasing similarity; q_self (optional) names a database row to skip per
 * query (~0 = none).  When fewer than k rows qualify, the remaining slots
 * hold id 0xFFFFFFFF and similarity -inf.  dims <= 256, k <= 32.  Host
 * buffers. */
int ep_knn_cosine(int device, uint64_t n_db, uint32_t dims, const float* db, uint64_t n_q, const float* q,
                  const uint64_t* q_self, uint32_t k, uint32_t* idx_out, float* sim_out);

/* NeighborhoodAligner.align (src/algos/alignment.rs:25-75, src/lib.rs:
 * 3040-3110): out[v] = (1 - a) * sum_j p_j emb[cols[j]] + a * emb[v] over
 * the first min(deg, max_neighbors) edges of v (max_neighbors 0 = all), p_j
 * the edge probabilities of the CDF weights w_cdf, a = alpha, or
 * min(1, 1 / ln(deg + 1)) when alpha < 0.  f32 arithmetic in the reference's
 * order.  A node without edges gets a * emb[v] (the reference indexes the
 * empty weight list).  emb / out: n_nodes x dims (<= 512).  Host buffers. */
int ep_align(int device, uint64_t n_nodes, const uint64_t* row_ptr, const uint32_t* cols, const float* w_cdf,
             uint32_t dims, const float* emb, float alpha, uint64_t max_neighbors, float* out);

/* Message of the last failing ep_embed_features / ep_align / ep_knn_cosine
 * call of this host thread. */
const char* ep_knn_last_error(void);

/* Measurement hook (no counterpart in the reference): CUDA-event time in ms
 * of the GPU kernel of this host thread's last ep_knn_cosine (the top-k
 * kernel) or ep_align call. */
float ep_knn_last_kernel_ms(void);

/* ---- host-side graph construction (src/graph.rs) --------------------- */

/* CSR::construct_from_edges (src/graph.rs:70-142): optional deduplication
 * (stable sort by (from, to), duplicate weights summed), nodes
 * 0..max(from,to).  rows_out holds max_node+2 entries, cols_out/w_out
 * n_edges entries; *n_nodes_out / *n_edges_out receive the sizes. */
int ep_csr_from_edges(uint64_t n_edges, const uint32_t* from, const uint32_t* to,
                      const float* w, int dedup, uint64_t* rows_out, uint32_t* cols_out,
                      float* w_out, uint64_t* n_nodes_out, uint64_t* n_edges_out);

/* CumCSR::convert (src/graph.rs:414-422, 664-691), in place. */
int ep_cdf_convert(uint64_t n_nodes, const uint64_t* rows, float* w);

/* ---- NodeEmbeddings text format (src/io.rs) -------------------------- */

/* EmbeddingWriter::stream (src/io.rs:44-76): rows i < n as lines
 * "<type>\t<name>\t[v0,...,v_{dims-1}]\n", each value the shortest decimal
 * that reads back to the same f32.  Types: with type_off, a byte buffer and
 * n+1 offsets; with type_off NULL, one NUL-terminated type for every row.
 * Names: with names, a byte buffer and n+1 offsets; with names NULL, the
 * decimal first_id + i.  Writes into out, which must hold the strings plus
 * n * (16 * dims + 25) bytes.  Returns the bytes written, or a negative
 * status. */
int64_t ep_format_embeddings(uint64_t n, uint32_t dims, const float* table, const char* types,
                             const uint64_t* type_off, const char* names, const uint64_t* name_off,
                             uint64_t first_id, char* out, uint64_t out_cap);

/* EmbeddingReader::load's line parser (src/io.rs:134-262) over a buffer of
 * whole lines "<type>\t<name>\t[v,...]" (blank lines skipped; values may be
 * padded with spaces and spell inf and NaN).  Counting call (values NULL):
 * returns the row count and sets *dims to the first row's width (0 when the
 * first row is malformed: a row holds at least one value).  Filling
 * call: *dims is the expected width; fills values (rows x dims) and, when
 * tok_off is given, 4 byte offsets per row (type begin/end, name begin/end),
 * and returns the row count.  A malformed line, or one of another width,
 * makes the filling call return EP_ERR_INVALID_ARG with *bad_line (when
 * given) set to its 1-based number among the non-blank lines (0 otherwise). */
int64_t ep_parse_embeddings(const char* buf, uint64_t len, uint32_t* dims, float* values, uint64_t* tok_off,
                            uint64_t* bad_line);

/* ---- Vocabulary and graph text files (src/vocab.rs, src/io.rs) --------- */

/* (node type, name) pairs -> dense ids in first-seen order (Vocab). */
typedef struct ep_vocab ep_vocab;
int ep_vocab_create(ep_vocab** out);
void ep_vocab_destroy(ep_vocab* v);
uint64_t ep_vocab_len(const ep_vocab* v);
/* Longest type + name of the vocabulary, in bytes. */
uint64_t ep_vocab_max_key(const ep_vocab* v);
/* Vocab::get_or_insert: the key's id, a new one when unseen. */
int64_t ep_vocab_intern(ep_vocab* v, const char* type, uint64_t type_len, const char* name, uint64_t name_len);
/* Vocab::get_node_id: the key's id, or -1. */
int64_t ep_vocab_find(const ep_vocab* v, const char* type, uint64_t type_len, const char* name, uint64_t name_len);
/* Interns n keys of buf given by 4 byte offsets each (type begin/end, name
 * begin/end, as ep_parse_embeddings writes them), in order; their ids to ids. */
int ep_vocab_intern_tokens(ep_vocab* v, const char* buf, const uint64_t* tok, uint64_t n, uint32_t* ids);
/* Bytes of the types and names of ids [lo, hi). */
int ep_vocab_range_bytes(const ep_vocab* v, uint64_t lo, uint64_t hi, uint64_t* type_bytes, uint64_t* name_bytes);
/* Types and names of ids [lo, hi) back to back, with hi-lo+1 offsets each. */
int ep_vocab_export(const ep_vocab* v, uint64_t lo, uint64_t hi, char* types, uint64_t* type_off, char* names,
                    uint64_t* name_off);

/* GraphReader::load's line step (src/io.rs:270-323) over a buffer of whole
 * lines "from_type\tfrom\tto_type\tto\tweight" (blank lines skipped):
 * interns from, then to, of each line in order and writes the ids and the
 * weight (1 when weighted is 0).  cap: capacity of src/dst/w in lines.
 * Returns the number of lines, or a negative status; for a malformed line
 * (not five fields, or a weight that is not a number) EP_ERR_INVALID_ARG
 * with *bad_line (when given) set to its 1-based number among the non-blank
 * lines, and nothing interned. */
int64_t ep_parse_edges(ep_vocab* v, const char* buf, uint64_t len, int weighted, uint32_t* src, uint32_t* dst,
                       float* w, uint64_t cap, uint64_t* bad_line);

/* Graph::save (src/lib.rs:414-430) for the rows of nodes [lo, hi): one line
 * per edge, the weight the edge's transition probability (difference of the
 * row's CDF) written as Rust's Display writes an f32.  Names come from v
 * (ids < n_nodes), or, with v NULL, node u is (anon_type, decimal u).  out
 * must hold (2 * longest type + name + 54) bytes per edge (the longest key
 * of v is ep_vocab_max_key).  Returns the bytes written into out, or a
 * negative status (also when out_cap is too small). */
int64_t ep_format_edges(const ep_vocab* v, const char* anon_type, uint64_t n_nodes, const uint64_t* rows,
                        const uint32_t* cols, const float* cdf, uint64_t lo, uint64_t hi, char* out, uint64_t out_cap);

/* FeaturePropagator::propagate (src/lib.rs:1695-1770, propagate_features in
 * src/algos/feat_propagation.rs:13-93) over the graph CSR (per-row CDF
 * weights) and the node -> feature CSR (fptr, fids).  Featureless nodes
 * receive up to k features of their neighbours; at most max_iters in-place
 * sweeps.  Writes the new node -> feature CSR to fptr_out (n+1) and fids_out
 * (capacity out_cap ids: fptr[n] + k * featureless nodes suffices).  Returns
 * the number of ids written, or a negative status. */
int64_t ep_propagate_features(uint64_t n, const uint64_t* rows, const uint32_t* cols, const float* cdf,
                              const uint64_t* fptr, const uint32_t* fids, uint32_t max_iters, uint32_t k,
                              float threshold, uint64_t* fptr_out, uint32_t* fids_out, uint64_t out_cap);

#ifdef __cplusplus
}
#endif
#endif
