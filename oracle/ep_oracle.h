/*
 * ep_oracle.h -- CPU restatement of cloverleaf's Embedding Propagation (EP)
 * training path.  TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke()
 * and bench.py's CPU baseline are the only callers.  The product path never
 * links or calls anything declared here.
 *
 * Parity status of this restatement:
 *   - CSR construction, deduplication and CDF weights are pinned by the
 *     reference's own unit tests (src/graph.rs:697-787), replayed in
 *     tests/test_oracle.py.
 *   - Euclidean distance and L2 normalisation are pinned by
 *     src/algos/ep/loss.rs:250-263.
 *   - EP loss, per-feature gradient extraction, batch reduction, Adam and the
 *     learning-rate schedule are UNPINNED: the reference is a Rust crate that
 *     cannot be built here (no cargo/rustc), its autograd dependency
 *     (simple_grad, git dependency with no pinned revision, Cargo.toml:20) is
 *     not vendored, and no reference test asserts EP loss or gradient values.
 *     They are restated from src/algos/ep/{mod,model,loss}.rs and
 *     src/algos/grad_utils/{optimizer,scheduler}.rs and cross-checked against
 *     an independent numpy restatement and central finite differences.
 */
#ifndef EP_ORACLE_H
#define EP_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Loss kinds (src/algos/ep/loss.rs:15-38).  RANK / RANKSPACE take tau in
 * gamma; PPR is the margin loss whose positive role is built from random-walk
 * end nodes (orc_train_cfg.ppr_restart_p; explicit samples give them as the
 * neighbour list with weight 1). */
enum {
    ORC_LOSS_MARGIN = 0,
    ORC_LOSS_STARSPACE = 1,
    ORC_LOSS_CONTRASTIVE = 2,
    ORC_LOSS_RANK = 3,
    ORC_LOSS_RANKSPACE = 4,
    ORC_LOSS_PPR = 5
};
/* Loss weighting (src/algos/ep/mod.rs:31-36). */
enum { ORC_LW_NONE = 0, ORC_LW_LOG = 1, ORC_LW_EXP = 2 };
/* Gradient extraction: reference = first finite occurrence of a feature
 * across roles wins (src/algos/ep/mod.rs:361-378); true = sum of all finite
 * occurrences (the derivative of the loss wherever it is defined). */
enum { ORC_GRAD_REFERENCE = 0, ORC_GRAD_TRUE = 1 };
/* Sample kinds (src/algos/utils.rs:165-217). */
enum { ORC_SAMPLE_ALL = 0, ORC_SAMPLE_FIXED = 1, ORC_SAMPLE_PROB = 2 };

typedef struct orc_loss_cfg {
    int32_t loss;
    float gamma;
    float neg_margin;     /* contrastive only */
    int32_t grad_mode;
    int32_t loss_weighting;
    float lw_exp;
    float feat_scalar;    /* s_u added to every node weight (1 for Sample::All) */
} orc_loss_cfg;

/* graph.rs:70-142.  Builds a CSR from an edge list.  rows_out must hold
 * max_node+2 entries, cols_out/w_out n_edges entries.  Returns 0. */
int orc_csr_from_edges(uint64_t n_edges, const uint64_t* from, const uint64_t* to,
                       const float* w, int dedup, uint64_t* rows_out,
                       uint64_t* cols_out, float* w_out,
                       uint64_t* n_nodes_out, uint64_t* n_edges_out);

/* graph.rs:414-422 with convert_edges_to_cdf graph.rs:664-691. */
void orc_cdf_convert(uint64_t n_nodes, const uint64_t* rows, float* w);

/* One EP batch from explicit samples (mod.rs:174-233 for one batch).
 * Roles per anchor a: 0 = the anchor itself (weight 1), 1 = its sampled
 * neighbours nbr[nbr_ptr[a]..nbr_ptr[a+1]) with base weights nbr_w,
 * 2..R+1 = negatives neg[a*R + i] (weight 1).  Every feature occurrence of a
 * node of base weight w counts w + cfg->feat_scalar (model.rs:257-278).
 * Outputs: loss_out[a] after weighting, status_out[a] (0 kept, 1 loss <= 0,
 * 2 NaN), grad_out (n_feat*d, caller zeroes) accumulates the batch gradient
 * and touched[f] marks rows present in the batch map.  Returns the number of
 * kept anchors. */
int orc_batch_f32(const uint64_t* fptr, const uint32_t* fids, uint32_t n_feat,
                  const float* table, uint32_t d, const uint64_t* graph_rows,
                  uint32_t B, const uint32_t* anchors, const uint32_t* nbr_ptr,
                  const uint32_t* nbr, const float* nbr_w, uint32_t R,
                  const uint32_t* neg, const orc_loss_cfg* cfg,
                  float* loss_out, int32_t* status_out, float* grad_out,
                  uint8_t* touched);
int orc_batch_f64(const uint64_t* fptr, const uint32_t* fids, uint32_t n_feat,
                  const float* table, uint32_t d, const uint64_t* graph_rows,
                  uint32_t B, const uint32_t* anchors, const uint32_t* nbr_ptr,
                  const uint32_t* nbr, const float* nbr_w, uint32_t R,
                  const uint32_t* neg, const orc_loss_cfg* cfg,
                  double* loss_out, int32_t* status_out, double* grad_out,
                  uint8_t* touched);

/* optimizer.rs:43-81: lazy Adam over touched rows, t = pass + 1. */
void orc_adam(float* table, float* m, float* v, uint32_t d, uint32_t n_feat,
              const float* grad, const uint8_t* touched, float lr, uint32_t pass);

/* scheduler.rs:120-137 CosDecay. */
float orc_lr_cos_decay(float min_alpha, float alpha, uint64_t warmup,
                       uint64_t max_steps, uint64_t cur_step);

typedef struct orc_train_cfg {
    float alpha;
    orc_loss_cfg loss;
    uint32_t negatives;
    uint32_t batch_size;
    uint32_t dims;
    uint32_t passes;
    uint64_t seed;
    int32_t max_nodes_kind;
    float max_nodes;
    int32_t max_features_kind;
    float max_features;
    float valid_pct;
    int32_t threads;        /* OpenMP threads, <= 0 means all */
    uint64_t max_batches;   /* stop after this many batches in total (0 = all) */
    uint32_t hard_negatives; /* random-walk negatives per anchor (node_sampler.rs:83-145) */
    float ppr_restart_p;    /* ORC_LOSS_PPR walk restart probability (loss.rs:166-187) */
} orc_train_cfg;

typedef struct orc_train_stats {
    double seconds;         /* wall time of the training passes */
    uint64_t anchors;       /* anchors processed */
    uint64_t batches;
    float last_train_loss;
    float last_valid_loss;
    double shuffle_seconds;  /* of `seconds`, spent shuffling the pass order (once per pass) */
    uint64_t steps_per_pass; /* batches of a full pass */
} orc_train_stats;

/* The whole learn_feature_embeddings loop (mod.rs:92-287): seeded init,
 * shuffles, batches processed in parallel (OpenMP), per-node hash maps,
 * first-occurrence extraction, per-batch merge, hogwild Adam.  table_io holds
 * n_feat*d floats: the initial table when init_given != 0, the result on
 * return. */
int orc_train(const uint64_t* rows, const uint32_t* cols, const float* wcdf,
              uint64_t n_nodes, const uint64_t* fptr, const uint32_t* fids,
              uint32_t n_feat, const orc_train_cfg* cfg, float* table_io,
              int init_given, orc_train_stats* stats);

#ifdef __cplusplus
}
#endif
#endif
