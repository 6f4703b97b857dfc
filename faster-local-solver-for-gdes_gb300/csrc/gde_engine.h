// gde_engine.h -- internal interface between the C-ABI layer and the kernels.
#pragma once
#include <cuda_runtime.h>

#include "gde_common.cuh"

namespace gde {

// Persistent push engine (push_engine.cu).
int engine_max_grid(int prec64, int W, int sms);
cudaError_t engine_launch(const PushArgs& a, int prec64, int W, int grid, cudaStream_t st);

// Column initialisation and result extraction (aux_kernels.cu).
struct InitCol {
    int tile, col;      // slot
    int seed;           // seed node
    double r0;          // residual at the seed
    double x0;          // solution at the seed (Chebyshev)
    double dx0;         // delta-x at the seed (Chebyshev)
    double push0;       // value pushed to every neighbour of the seed (Chebyshev), 0 = none
};
cudaError_t init_columns(const PushArgs& a, int prec64, int W, const InitCol* d_cols, int ncols, cudaStream_t st);

struct ExtractCol {
    int tile, col;      // slot
    int64_t out_row;    // row of the output matrices
    int seed;           // node whose solution gets `seed_add` (Katz GD: -1)
    double seed_add;
    double scale;       // solution divided by this (HK: e^tau), 1 otherwise
    int r_levels;       // 2: HK residual [2, n] output, 1 otherwise
};
cudaError_t extract_columns(const PushArgs& a, int prec64, int W, const ExtractCol* d_cols, int ncols, void* x_out,
                            void* r_out, int out64, int64_t ld_out, int64_t n, int clear, cudaStream_t st);

// Plain single-query baseline (plain.cu).
struct PlainWork {
    float *xt, *rt, *tmp, *sp, *eps_vec, *degf;
    int32_t *queue, *nz;
    int *d_count;
    double *d_oper;
    int *h_count;      // pinned
};
int plain_ppr_local(const DevGraph& g, PlainWork& w, int seed, double alpha, double eps, double* oper,
                    int* rounds, cudaStream_t st);

// Row permutation between caller and internal node order (aux_kernels.cu):
// to_internal: dst[perm[u]] = src[u]; else dst[u] = src[perm[u]] (row strides sld, dld).
cudaError_t permute_rows(const void* src, int64_t sld, void* dst, int64_t dld, const int32_t* perm, int64_t n,
                         int64_t F, int elem, int to_internal, cudaStream_t st);

// Entry permutation within rows (aux_kernels.cu): per row r < rows,
// dst[r * dld + u] = src[r * sld + perm[u]] for u < n (internal -> caller order).
cudaError_t permute_entries(const void* src, int64_t sld, void* dst, int64_t dld, const int32_t* perm, int64_t n,
                            int64_t rows, int elem, cudaStream_t st);

// Served solutions kept per query ({x, Kahan term} slabs with tile offset
// xtile, internal node order) -> caller-order rows out[q * ld_out + u]
// (aux_kernels.cu); the Katz seed entry gets -1 (kinds null: seed_add) and
// heat-kernel rows are divided by hk_scale = e^tau.  With iperm (internal ->
// caller) the slabs are read in internal order and scattered into the rows
// (device rows); else the rows are gathered through perm (null: no relabel).
cudaError_t query_rows(const float* XI, int64_t xtile, const int32_t* perm, const int32_t* iperm, int64_t n,
                       int64_t nq, const int32_t* seed_int, const int32_t* kinds, double seed_add, double hk_scale,
                       void* out, int out64, int64_t ld_out, cudaStream_t st);

// One touched node's degree tables after an edge batch.
struct NodeTables {
    int32_t id, len;
    double degd, nf, tf;  // degree; InstantGNN d^(1-beta), d^beta
};
// Write the tables of nn touched nodes (nfac null: degrees only).
cudaError_t node_tables(int64_t nn, const NodeTables* rec, int32_t* row_len, double* degd, float* degf, double* nfac,
                        double* tfac, float* tfac_f, cudaStream_t st);

// Graph helpers (aux_kernels.cu).
cudaError_t graph_apply_entries(int32_t* col, const int64_t* pos, const int32_t* val, int64_t k, cudaStream_t st);

}  // namespace gde
