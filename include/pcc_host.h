/*
 * pcc_host.h -- C ABI of libpcc_host.so: host-side utilities around the GPU
 * clusterer (synthetic graph generators, GBBS adjacency-graph I/O, the
 * text-format ClustererConfig parser and clustering output).
 *
 * Graphs returned here are owned by the library; free them with
 * pcch_graph_free.  offsets/neighbors/weights use the same symmetric CSR
 * layout as pcc_gb300.h; weights is NULL for unit-weight graphs and truth
 * (planted communities) is NULL when the generator has none.
 */
#ifndef PCC_HOST_H_
#define PCC_HOST_H_

#include <stddef.h>
#include <stdint.h>

#include "pcc_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pcch_graph {
  uint32_t n;
  uint64_t m;
  uint64_t* off;     /* offsets, n + 1 */
  uint32_t* nbr;     /* neighbour ids, m */
  float* w;          /* weights, m, or NULL */
  uint32_t* truth;   /* planted community per vertex, or NULL */
} pcch_graph;

void pcch_graph_free(pcch_graph* g);

/* Stochastic block model (uniform block assignment, p_in / p_out). */
pcch_graph* pcch_gen_sbm(uint32_t n, uint32_t blocks, double p_in, double p_out, uint64_t seed);
/* RMAT with 2^scale vertices and edge_factor * 2^scale samples. */
pcch_graph* pcch_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed);
/* LFR-like planted partition (power-law degrees and community sizes). */
pcch_graph* pcch_gen_lfr(uint32_t n, double mean_degree, uint32_t dmax, double tau1, uint32_t cmin, uint32_t cmax,
                         double tau2, double mu, double w_lo, double w_hi, uint64_t seed);

/*
 * Text-format ClustererConfig (clustering/config.proto:94-197) -> pcc_config,
 * as TextFormat::ParseFromString in cluster-in-memory_main.cc:256-264.
 * config_case: 0 unset, 1 parameter_string, 4 affinity, 7 correlation.
 * err (may be NULL) receives the parse error message.  Returns a status code.
 */
int32_t pcch_parse_config(const char* text, pcc_config* out, int32_t* config_case, char* err, size_t err_len);

/*
 * GBBS adjacency text file ("AdjacencyGraph" / "WeightedAdjacencyGraph"),
 * as gbbs_io::read_(un)weighted_symmetric_graph in cluster-in-memory_main.cc:
 * 286-306.  Returns NULL and sets *status on error.  All-one weights are
 * dropped (unit-weight graph).
 */
pcch_graph* pcch_read_gbbs(const char* path, int32_t float_weighted, int32_t* status);

/*
 * CompareCommunities (cluster-in-memory_main.cc:167-222) of a clustering
 * given as labels[n] (cluster index per node) against a communities file
 * (tab-separated node ids, one community per line).  out6 = {avg precision,
 * avg recall, number of clusters, min size, max size, avg size}.
 */
int32_t pcch_compare_communities(const char* communities_path, uint32_t n, const uint32_t* labels, double* out6);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* PCC_HOST_H_ */
