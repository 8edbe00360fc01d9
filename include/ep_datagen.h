/*
 * ep_datagen.h -- seeded synthetic workloads for the EP trainer.
 *
 * No counterpart in the reference: cloverleaf ships no EP benchmark data (its
 * Pinterest example data is not part of the repository), so the tests and the
 * benchmark build planted-community (SBM) and power-law (Chung-Lu) graphs with
 * hashed-token features here.  Outputs are plain CSR arrays in the layout of
 * ep_upload_graph / ep_upload_features; every generator is deterministic in
 * its seed and independent of the number of host threads.
 *
 * Two-call protocol: call with NULL output pointers to get the sizes, then
 * again with buffers of those sizes (the second call regenerates the same
 * data from the seed).  Every function returns 0 on success and -1 for an
 * invalid argument.
 *
 * Exported by libep_datagen.so, a host-only library separate from the
 * trainer's libep_gb300.so.
 */
#ifndef EP_DATAGEN_H
#define EP_DATAGEN_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Undirected stochastic block model: n nodes in `blocks` equal contiguous
 * communities (community of node i = i * blocks / n), expected intra-degree
 * k_in and inter-degree k_out, weight 1, both directions stored, rows sorted.
 * A node left isolated gets one edge to a random member of its community.
 * community_out (n entries, optional) receives each node's community. */
int epg_sbm(uint64_t n, uint32_t blocks, double k_in, double k_out, uint64_t seed,
            uint64_t* row_ptr, uint32_t* cols, float* w, uint32_t* community_out,
            uint64_t* n_edges_out);

/* Token features for SBM nodes: each node draws tok_min..tok_max tokens
 * (uniform count); a token comes from its community's `sub_vocab` tokens with
 * probability p_local, else from a global vocabulary of `global_vocab`
 * tokens; it is hashed into 2^slot_bits slots.  Slots are interned to dense
 * feature ids in first-seen order (node order, then token order), as
 * FeatureStore::set_features does (src/feature_store.rs:36-48).
 * slot_of_feature (optional, n_feat_out entries) maps feature id -> slot. */
int epg_sbm_tokens(uint64_t n, const uint32_t* community, uint32_t tok_min, uint32_t tok_max,
                   uint32_t sub_vocab, uint32_t global_vocab, double p_local, uint32_t slot_bits,
                   uint64_t seed, uint64_t* fptr, uint32_t* fids, uint32_t* slot_of_feature,
                   uint64_t* n_fids_out, uint32_t* n_feat_out);

/* Chung-Lu graph: expected degrees follow a power law with the given
 * exponent, clipped to [1, max_degree] with the scale recalibrated so the
 * clipped mean is mean_degree; round(n * mean_degree / 2) undirected edge
 * draws with endpoints proportional to the expected degrees, self loops and
 * duplicates dropped, both directions stored, rows sorted.  bipartite != 0
 * draws one endpoint from [0, n/2) and the other from [n/2, n).  Weights are
 * 1, or uniform in [w_lo, w_hi] when w_hi > w_lo.  Nodes left isolated get one
 * edge.  Multithreaded; deterministic in seed. */
int epg_chung_lu(uint64_t n, double exponent, double mean_degree, double max_degree,
                 int bipartite, float w_lo, float w_hi, uint64_t seed, uint64_t* row_ptr,
                 uint32_t* cols, float* w, uint64_t* n_edges_out);

/* Zipf features: count per node Poisson(lambda) clipped to [cmin, cmax] (or
 * uniform in [cmin, cmax] when lambda <= 0); each feature an independent
 * Zipf(s) draw over n_slots slot ids, which are used as feature ids
 * (n_feat = n_slots). */
int epg_zipf_features(uint64_t n, double lambda, uint32_t cmin, uint32_t cmax, double s,
                      uint32_t n_slots, uint64_t seed, uint64_t* fptr, uint32_t* fids,
                      uint64_t* n_fids_out);

#ifdef __cplusplus
}
#endif
#endif
