// gde_internal.h -- the library's context and resident-graph records, shared
// by the host translation units (not part of the C ABI: callers only see the
// opaque gde_ctx / gde_graph handles of include/gde.h).
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "gde_common.cuh"
#include "gde_engine.h"

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

constexpr int kDefaultMaxRounds = 100000;

struct gde_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sms = 0;
    std::string err;
    gde::GridBarrier* bar = nullptr;
    int* derr = nullptr;
    gde::LaunchStats* dstats = nullptr;
    gde::LaunchStats* hstats = nullptr;  // pinned
    gde::TileState* hts = nullptr;       // pinned scratch
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::map<std::string, DevBuf> ws;
    std::vector<int> stamp;         // per-tile stamp bases (valid while "mark" is allocated)
    gde::PlainWork plain{};
    int64_t plain_n = -1;
    // opt-in push-kernel phase trace (gde_ctx_trace)
    unsigned long long* trace = nullptr;
    int trace_iters = 0;
    int trace_grid = 0;
    // bounded device waits: polls before a wait gives up (0: the defaults);
    // set by gde_ctx_set_wait_limit to exercise the GDE_EHANG paths
    int64_t wait_limit = 0;
};

struct gde_graph {
    gde_ctx* ctx = nullptr;
    gde::DevGraph g{};
    int64_t* row_ptr = nullptr;
    int32_t* col = nullptr;
    int32_t* row_len = nullptr;
    float* degf = nullptr;
    double* degd = nullptr;
    double* nfac = nullptr;
    double* npush = nullptr;
    double* tfac = nullptr;
    float* tfac_f = nullptr;
    double ign_beta = NAN;
    // d^(1-beta), d^beta for integer degrees 0..pw_max (InstantGNN tables by
    // table lookup after edge insertions on the device), for beta = pw_beta
    double* pw1 = nullptr;
    double* pwb = nullptr;
    int64_t pw_max = -1;
    double pw_beta = NAN;
    // greedy proper colouring (internal ids), built on first use by the LocalSOR engine
    std::vector<int32_t> h_color;
    int ncolors = 0;
    std::vector<int64_t> h_indptr;
    std::vector<int64_t> h_len;
    std::vector<int32_t> edit_last;  // per node, -1 between edge batches (scratch of the device edit)
    std::vector<double> h_deg;
    bool deg_is_len = true;
    // Static graphs are stored relabelled by descending degree: push targets
    // are hit in proportion to their degree, so the hot part of every
    // residual vector is a short prefix that stays in L2.  h_perm maps a
    // caller id to the internal id; every API id stays the caller's.
    bool relabeled = false;
    std::vector<int32_t> h_perm;
    int32_t* perm_d = nullptr;
    int32_t* iperm_d = nullptr;  // internal id -> caller id (relabelled graphs)
    double dmax = -1.0;          // largest degree (< 0: not computed since the last edit)
    double lam_max_est = NAN;    // adjacency spectral radius from gde_katz_spectral_bounds (NaN: none)
    uint32_t* col_deg = nullptr;
    gde::NodeRec* rec = nullptr;
    int32_t node_in(int64_t u) const { return relabeled ? h_perm[u] : (int32_t)u; }
};
