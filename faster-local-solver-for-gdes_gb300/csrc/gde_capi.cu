// gde_capi.cu -- C ABI: contexts, resident graphs, tile workspaces, solves.
//
// Host orchestration of the GB300 push engine.  A solve groups its queries
// into node x column tiles, initialises the tiles' seeds, runs every tile to
// completion in one cooperative persistent launch, and extracts the
// per-query solution rows.  All reference-facing semantics (thresholds,
// operation counts, the Chebyshev and heat-kernel coefficient tables) are
// computed here in FP64 exactly as the reference computes them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "gde_common.cuh"
#include "gde_engine.h"

using namespace gde;

#include "gde_internal.h"

// sor_engine.cu: the InstantGNN push with relaxation omega != 1
int gde_internal_sor_feature_push(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t F, void* Pm, void* Rm,
                                  int64_t ld, double eps, const int32_t* d_cand, int64_t ncand, double* oper_out,
                                  gde_stats* stats);



namespace {

int fail(gde_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(gde_ctx* c, cudaError_t e, const char* where) {
    return fail(c, GDE_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                               \
    do {                                                       \
        cudaError_t e__ = (call);                              \
        if (e__ != cudaSuccess) return cuda_fail(ctx, e__, #call); \
    } while (0)

// Device workspace buffer `name` of at least `bytes` (grown on demand).
void* wsget(gde_ctx* ctx, const std::string& name, size_t bytes, bool* fresh = nullptr) {
    DevBuf& b = ctx->ws[name];
    if (fresh) *fresh = false;
    if (b.bytes >= bytes && b.p) return b.p;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    size_t want = std::max<size_t>(bytes, 256);
    if (cudaMalloc(&b.p, want) != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        return nullptr;
    }
    b.bytes = want;
    if (fresh) *fresh = true;
    return b.p;
}

void ws_release_all(gde_ctx* ctx) {
    for (auto& kv : ctx->ws)
        if (kv.second.p) cudaFree(kv.second.p);
    ctx->ws.clear();
}

int64_t estimate_n(double t, double eps) {
    // hk_solver.py:15-48 (estimate_coefficient / estimate_n) in the same FP64 order
    double kf = std::ceil(t - 1);
    int64_t k = (int64_t)kf;
    double t0 = t;
    if (k != 0)
        for (int64_t i = 0; i < k; i++) t0 = t0 * (t / (double)(i + 2));
    double cur_est = t0 * ((kf + 2.) / (kf + 2. - t));
    if (cur_est < eps * std::exp(t)) return k;
    int64_t est_k = k;
    for (int64_t i = k; i < 1000 * (k + 1); i++) {
        double tmp = ((kf + 2. - t) * t / std::pow(kf + 2., 2.)) * ((kf + 3.) / (kf + 3. - t));
        cur_est = cur_est * tmp;
        est_k += 1;
        if (cur_est < eps * std::exp(t)) return est_k;
    }
    return est_k;
}

struct Defaults {
    // every piece of push work is at most 8 dependent warp iterations (W = 1):
    // short rows one lane each, medium rows one warp each, long rows split
    // into warp-sized chunks
    int small_max = 8, med_max = 256, chunk = 256, dense_div = 2;
};

void fill_tuning(const gde_params* p, PushArgs& a) {
    Defaults d;
    a.small_max = p->small_max > 0 ? p->small_max : d.small_max;
    a.med_max = p->med_max > 0 ? p->med_max : d.med_max;
    if (a.med_max < a.small_max) a.med_max = a.small_max;
    a.chunk = p->chunk > 0 ? p->chunk : d.chunk;
    a.dense_div = p->dense_div > 0 ? p->dense_div : d.dense_div;
    a.max_rounds = p->max_rounds > 0 ? p->max_rounds : kDefaultMaxRounds;
    a.allow_dense = 1;
}

// Katz near its convergence radius (alpha * lambda_max close to 1) computes
// in FP64 whatever precision was asked: its series then converges slowly
// and FP32 residuals lose the stopping rule's accuracy.  The largest degree
// bounds lambda_max from above and settles most calls; when it cannot, the
// graph's Lanczos estimate (gde_katz_spectral_bounds, run once and cached
// until the graph is edited) decides.
constexpr double kKatzFp64Ratio = 0.9;
int katz_compute_prec(gde_ctx* ctx, gde_graph* G, const gde_params* p) {
    if (p->kind != KIND_KATZ || p->prec == GDE_FP64) return p->prec;
    if (G->dmax < 0.0) {
        double m = 0.0;
        for (double d : G->h_deg) m = std::max(m, d);
        G->dmax = m;
    }
    if (p->alpha * G->dmax < kKatzFp64Ratio) return p->prec;
    if (std::isnan(G->lam_max_est)) {
        double lmax = 0.0, lmin = 0.0;
        if (gde_katz_spectral_bounds(ctx, G, p->alpha, 300, 1e-8, &lmax, &lmin, nullptr, nullptr) != GDE_OK) {
            G->lam_max_est = G->dmax;  // no estimate: keep the bound
            ctx->err.clear();
        }
    }
    return (p->alpha * G->lam_max_est >= kKatzFp64Ratio) ? GDE_FP64 : p->prec;
}

bool valid_w(int W) { return W == 1 || W == 2 || W == 4 || W == 8 || W == 16 || W == 32; }

// Workspace for `ntiles` tiles of width W over n nodes.
struct TileWs {
    PushArgs a{};
    size_t elem = 0;
};

int alloc_tiles(gde_ctx* ctx, gde_graph* G, int ntiles, int W, int prec64, bool need_r2, bool need_dx,
                bool own_slabs, bool kahan, TileWs& tw) {
    const int64_t n = G->g.n;
    const size_t es = prec64 ? 8 : 4;
    const size_t slab = (size_t)ntiles * n * W * es;
    PushArgs& a = tw.a;
    a.g = G->g;
    a.ntiles = ntiles;
    // one-column FP32 Kahan slabs interleave the solution and its Kahan term
    // as {x, c} pairs, so a frontier node's update touches one sector
    const bool inter = own_slabs && kahan && !prec64 && W == 1;
    if (own_slabs) {
        a.ld = W;
        a.tile_stride = (int64_t)n * W;
        a.R = wsget(ctx, "R", slab);
        a.X = wsget(ctx, "X", inter ? 2 * slab : slab);
        if (!a.R || !a.X) return fail(ctx, GDE_ENOMEM, "device memory exhausted (residual/solution slabs)");
        a.R2 = need_r2 ? wsget(ctx, "R2", slab) : nullptr;
        a.DX = need_dx ? wsget(ctx, "DX", slab) : nullptr;
        if ((need_r2 && !a.R2) || (need_dx && !a.DX)) return fail(ctx, GDE_ENOMEM, "device memory exhausted (slabs)");
    }
    a.XC = nullptr;
    a.kahan = 0;
    a.xld = 0;
    a.xtile = 0;
    if (kahan && !prec64 && own_slabs) {
        if (inter) {
            a.XC = (float*)a.X + 1;
            a.xld = 2;
            a.xtile = 2 * n;
        } else {
            a.XC = (float*)wsget(ctx, "XC", (size_t)ntiles * n * W * 4);
            if (!a.XC) return fail(ctx, GDE_ENOMEM, "device memory exhausted (Kahan slab)");
        }
        a.kahan = 1;
    }
    a.P = wsget(ctx, "P", slab);
    a.cand = (int32_t*)wsget(ctx, "cand", (size_t)ntiles * 2 * n * 4);
    a.bsmall = (PushItem*)wsget(ctx, "items", (size_t)ntiles * n * sizeof(PushItem));
    bool fresh = false;
    a.mark = (int32_t*)wsget(ctx, "mark", (size_t)ntiles * n * 4, &fresh);
    if (!a.P || !a.cand || !a.bsmall || !a.mark)
        return fail(ctx, GDE_ENOMEM, "device memory exhausted (frontier lists)");
    if (fresh) {
        CK(cudaMemsetAsync(a.mark, 0xff, ctx->ws["mark"].bytes, ctx->stream));
        ctx->stamp.assign(ctx->ws["mark"].bytes / 4 / std::max<int64_t>(n, 1) + 1, 0);
    }
    if ((int)ctx->stamp.size() < ntiles) ctx->stamp.resize(ntiles, 0);
    {
        // A tile's marks live at mark + t * n, so a graph of another size maps
        // tile t onto marks another tile wrote.  Every tile therefore starts
        // past the largest stamp any tile has used (marks are compared for
        // equality); near the int range the marks are reset instead.
        int base = *std::max_element(ctx->stamp.begin(), ctx->stamp.end());
        if (base > (1 << 30)) {
            CK(cudaMemsetAsync(a.mark, 0xff, ctx->ws["mark"].bytes, ctx->stream));
            base = 0;
        }
        std::fill(ctx->stamp.begin(), ctx->stamp.end(), base);
    }
    tw.elem = es;
    a.tp = (TileParams*)wsget(ctx, "tp", (size_t)ntiles * sizeof(TileParams));
    a.ts = (TileState*)wsget(ctx, "ts", (size_t)ntiles * sizeof(TileState));
    a.cs = (ColState*)wsget(ctx, "cs", (size_t)ntiles * W * sizeof(ColState));
    if (!a.tp || !a.ts || !a.cs) return fail(ctx, GDE_ENOMEM, "device memory exhausted (tile state)");
    a.stats = ctx->dstats;
    a.trace = ctx->trace;
    a.trace_iters = ctx->trace ? ctx->trace_iters : 0;
    a.spin_limit = (unsigned long long)std::max<int64_t>(ctx->wait_limit, 0);
    a.bar = ctx->bar;
    a.err = ctx->derr;
    return GDE_OK;
}

int alloc_large(gde_ctx* ctx, gde_graph* G, int ntiles, TileWs& tw) {
    PushArgs& a = tw.a;
    int64_t cap = G->g.cap;
    a.large_cap = cap / std::max(a.chunk, 1) + cap / std::max(a.med_max, 1) + 64;
    a.blarge = (PushItem*)wsget(ctx, "blarge", (size_t)ntiles * a.large_cap * sizeof(PushItem));
    if (!a.blarge) return fail(ctx, GDE_ENOMEM, "device memory exhausted (chunk list)");
    return GDE_OK;
}

// Run the persistent engine until every tile is done (or max_rounds).
int run_engine(gde_ctx* ctx, PushArgs& a, int prec64, int W, gde_stats* st, double* kernel_ms) {
    int grid = engine_max_grid(prec64, W, ctx->sms);
    if (grid <= 0) return fail(ctx, GDE_ECUDA, "push kernel does not fit on the device");
    if (a.serve && a.queue.sp_blocks > grid / 2) a.queue.sp_blocks = grid / 2;  // at least half the grid stays dense
    const int dense_grid = grid - (a.serve ? a.queue.sp_blocks : 0);
    if (a.groups > dense_grid) a.groups = dense_grid;  // every group holds at least one block
    CK(cudaMemsetAsync(ctx->bar, 0, kMaxGroups * sizeof(GridBarrier), ctx->stream));
    CK(cudaMemsetAsync(ctx->derr, 0, sizeof(int), ctx->stream));
    CK(cudaMemsetAsync(ctx->dstats, 0, sizeof(LaunchStats), ctx->stream));
    if (ctx->trace) {
        CK(cudaMemsetAsync(ctx->trace, 0, (size_t)ctx->trace_iters * grid * kTracePoints * 8, ctx->stream));
        ctx->trace_grid = grid;
    }
    if (!a.serve) a.round_budget = a.max_rounds + 1;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    cudaError_t e = engine_launch(a, prec64, W, grid, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cooperative launch of the push kernel");
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, ctx->derr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(ctx->hstats, ctx->dstats, sizeof(LaunchStats), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    *kernel_ms += ms;
    if (st) {
        st->rounds += (int64_t)ctx->hstats->rounds;
        st->dense_rounds += (int64_t)ctx->hstats->dense_rounds;
        st->union_vol += ctx->hstats->union_vol;
        st->col_vol += ctx->hstats->col_vol;
        st->union_nodes += ctx->hstats->union_nodes;
        st->col_nodes += ctx->hstats->col_nodes;
        st->check_ms += (double)ctx->hstats->check_ns * 1e-6;
        st->prep_ms += (double)ctx->hstats->prep_ns * 1e-6;
        st->scatter_ms += (double)ctx->hstats->scatter_ns * 1e-6;
        st->sparse_queries += (int64_t)ctx->hstats->sp_done;
        st->sparse_overflows += (int64_t)ctx->hstats->sp_ovf;
    }
    if (herr != 0) {
        // The launch stopped part-way: its marks may carry stamps the next
        // launch would reuse, so every mark starts over (stamps from 0).
        auto it = ctx->ws.find("mark");
        if (it != ctx->ws.end() && it->second.p) {
            CK(cudaMemsetAsync(it->second.p, 0xff, it->second.bytes, ctx->stream));
            CK(cudaStreamSynchronize(ctx->stream));
        }
        std::fill(ctx->stamp.begin(), ctx->stamp.end(), 0);
        return fail(ctx, herr, "a device-side wait ran out of iterations (grid barrier)");
    }
    return GDE_OK;
}

// Chebyshev coefficient tables (ppr_solver.py:608-609, :636-637; katz_solver.py:366-368)
std::vector<double> cheby_table(int kind, double alpha, double l_max, double mu_min, int rounds) {
    std::vector<double> t;
    if (kind == KIND_KATZ) {
        double delta = (l_max - mu_min) / (l_max + mu_min);
        t.resize(2 * (size_t)rounds);
        for (int i = 0; i < rounds; i++) {
            delta = 1. / (2. * ((l_max + mu_min) / (l_max - mu_min)) - delta);
            t[2 * i] = 4. * delta / (l_max - mu_min);
            t[2 * i + 1] = (1. - 2. * delta * (l_max + mu_min) / (l_max - mu_min));
        }
    } else {
        double delta = (1. - alpha);
        t.resize(rounds);
        for (int i = 0; i < rounds; i++) {
            delta = 1. / (2. / (1. - alpha) - delta);
            t[i] = 2. * delta / (1. - alpha);
        }
    }
    return t;
}

// psi table of hk_sor_queue (hk_solver.py:226-229)
std::vector<double> psi_table(double tau, int64_t N) {
    std::vector<double> psi(N + 2, 1.0);
    psi[N] = 1.;
    for (int64_t i = N - 1; i >= 0; i--) psi[i] = psi[i + 1] * tau / ((double)i + 1.) + 1.;
    return psi;
}

int upload_ign_tables(gde_ctx* ctx, gde_graph* G, double beta) {
    const int64_t n = G->g.n;
    std::vector<double> nf(n), tf(n);
    std::vector<float> tff(n);
    for (int64_t u = 0; u < n; u++) {
        double d = G->h_deg[u];
        nf[u] = std::pow(d, 1 - beta);  // np.power(degree, 1 - beta), InstantGNN.py:57
        tf[u] = std::pow(d, beta);      // degree[v] ** beta, InstantGNN.py:31
        tff[u] = (float)tf[u];
    }
    if (!G->nfac) {
        CK(cudaMalloc(&G->nfac, n * 8));
        CK(cudaMalloc(&G->tfac, n * 8));
        CK(cudaMalloc(&G->tfac_f, n * 4));
    }
    CK(cudaMemcpyAsync(G->nfac, nf.data(), n * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(G->tfac, tf.data(), n * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(G->tfac_f, tff.data(), n * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    G->npush = G->nfac;
    G->g.nfac = G->nfac;
    G->g.npush = G->nfac;
    G->g.tfac = G->tfac;
    G->g.tfac_f = G->tfac_f;
    G->ign_beta = beta;
    return GDE_OK;
}

int upload_degrees(gde_ctx* ctx, gde_graph* G) {
    const int64_t n = G->g.n;
    std::vector<int32_t> len(n);
    std::vector<float> df(n);
    double vol = 0;
    for (int64_t u = 0; u < n; u++) {
        len[u] = (int32_t)G->h_len[u];
        df[u] = (float)G->h_deg[u];
        vol += G->h_deg[u];
    }
    CK(cudaMemcpyAsync(G->row_len, len.data(), n * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(G->degd, G->h_deg.data(), n * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(G->degf, df.data(), n * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    G->g.vol = vol;
    int exact = 1;
    for (int64_t u = 0; u < n; u++)
        if ((double)df[u] != G->h_deg[u]) { exact = 0; break; }
    G->g.degf_exact = exact;
    return GDE_OK;
}

constexpr int64_t kHubLen = 64;  // rows longer than this are hubs (warp-combined atomics)

// Static graphs: node records {row start, length, degree} and, when every
// degree is an exact integer, column words carrying the target's degree in
// the bits above the node id.  A graph that is edited later never gets them.
int build_static_records(gde_ctx* ctx, gde_graph* G, const int32_t* col) {
    const int64_t n = G->g.n, cap = G->g.cap;
    std::vector<NodeRec> rec(n);
    for (int64_t u = 0; u < n; u++) {
        rec[u].rp = G->h_indptr[u];
        rec[u].len = (int)G->h_len[u];
        rec[u].degf = (float)G->h_deg[u];
    }
    if (cudaMalloc(&G->rec, n * sizeof(NodeRec)) != cudaSuccess) {
        cudaGetLastError();
        G->rec = nullptr;
        return fail(ctx, GDE_ENOMEM, "device memory exhausted (node records)");
    }
    CK(cudaMemcpyAsync(G->rec, rec.data(), n * sizeof(NodeRec), cudaMemcpyHostToDevice, ctx->stream));
    G->g.rec = G->rec;
    int bits = 1;
    while (((int64_t)1 << bits) < n) bits++;
    const int dbits = 32 - bits;
    if (G->g.degf_exact && dbits >= 4 && cap > 0) {
        const uint32_t esc = (1u << dbits) - 1u;
        std::vector<uint32_t> packed(cap);
        for (int64_t j = 0; j < cap; j++) {
            const int32_t v = col[j];
            const double d = G->h_deg[v];
            const uint32_t code = (d >= 0.0 && d < (double)esc && d == std::floor(d)) ? (uint32_t)d : esc;
            packed[j] = (uint32_t)v | (code << bits);
        }
        if (cudaMalloc(&G->col_deg, cap * sizeof(uint32_t)) != cudaSuccess) {
            cudaGetLastError();
            G->col_deg = nullptr;
            return fail(ctx, GDE_ENOMEM, "device memory exhausted (packed columns)");
        }
        CK(cudaMemcpyAsync(G->col_deg, packed.data(), cap * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
        G->g.col_deg = G->col_deg;
        G->g.idx_bits = bits;
        G->g.deg_esc = esc;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return GDE_OK;
}

// Served solve of PPR / Katz local GD: `slots` single-column tiles cycle
// through a device queue of the nq queries inside one persistent launch.  A
// finished query's solution row is written (caller node order) and its slot
// cleared by the kernel itself, and the next query admitted -- continuous
// batching, so only `slots` residual vectors are ever live and they stay
// L2-resident.  arrival_ms (may be null): query q is not admitted before
// arrival_ms[q] after the launch starts; latency is then measured from it.
// kinds / alphas (may be null): a mixed queue of PPR, Katz and heat-kernel
// queries, each slot taking the kind of the query it admits.
// budget_bytes > 0 caps the slot count so the slots' vectors fit in it.

// Served FP32 slots keep the residual of at most this many highest-degree
// nodes in FP64 (the graph's hub prefix: rows longer than kHubLen).
constexpr int64_t kRhMax = 1 << 16;

int64_t served_slot_bytes(int64_t n, int64_t cap, int prec64, bool hk, const PushArgs& tun, int64_t hub_cut) {
    const int64_t es = prec64 ? 8 : 4;
    const int64_t large_cap = cap / std::max(tun.chunk, 1) + cap / std::max(tun.med_max, 1) + 64;
    return n * es * (3 + (hk ? 1 : 0)) + (prec64 ? 0 : n * 4 + std::min(hub_cut, kRhMax) * 8) + n * 4 * 3 +
           n * (int64_t)sizeof(PushItem) + large_cap * (int64_t)sizeof(PushItem);
}

int solve_served(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t nq, const int32_t* seeds,
                 const double* eps, const double* arrival_ms, void* x_out, void* r_out, int out64, int out_mem,
                 int64_t ld_out, double* oper_out, int32_t* rounds_out, float* lat_ms_out, gde_stats* stats,
                 const int32_t* kinds = nullptr, const double* alphas = nullptr, double budget_bytes = 0.0) {
    const int64_t n = G->g.n;
    const int kind = p->kind;
    const int prec64 = (p->prec == GDE_FP64);
    if (nq >= (int64_t)1 << 31) return fail(ctx, GDE_EINVAL, "too many queries");
    bool any_hk = false;
    if (kinds)
        for (int64_t q = 0; q < nq; q++) any_hk |= (kinds[q] == KIND_HK);
    int S = p->slots > 0 ? p->slots : 32;
    S = (int)std::min<int64_t>(std::min<int64_t>(S, nq), 512);
    PushArgs base{};
    fill_tuning(p, base);
    if (budget_bytes > 0.0) {
        // admission by memory budget: only as many slots as fit
        const int64_t per = served_slot_bytes(n, G->g.cap, prec64, any_hk, base, G->g.hub_cut);
        const int64_t fit = (int64_t)(budget_bytes / (double)per);
        if (fit < 1) return fail(ctx, GDE_ENOMEM, "the HBM budget does not hold one query slot");
        S = (int)std::min<int64_t>(S, fit);
    }
    TileWs tw;
    tw.a = base;
    int rc = alloc_tiles(ctx, G, S, 1, prec64, any_hk, false, true, !prec64, tw);
    if (rc != GDE_OK) return rc;
    PushArgs& a = tw.a;
    a.small_max = base.small_max; a.med_max = base.med_max; a.chunk = base.chunk;
    a.dense_div = base.dense_div; a.max_rounds = base.max_rounds; a.allow_dense = base.allow_dense;
    // Independent slot groups, each behind its own barrier.  The default is
    // one group per slot for PPR-only queues (measured best on the 2.36M- and
    // 100k-node PPR workloads: a slot's rounds wait only for the ~12 blocks
    // working on it, and the groups keep the memory system busy while one
    // waits), and one group per 8 slots when the queue holds Katz or
    // heat-kernel queries, whose frontiers span much of the graph and want
    // more blocks each (measured on the R-MAT mix: +25% saturation and a
    // 7x lower p99 at light load than one group per slot).
    bool wide = (kind == KIND_KATZ || kind == KIND_HK);
    if (kinds)
        for (int64_t q = 0; q < nq && !wide; q++) wide = (kinds[q] == KIND_KATZ || kinds[q] == KIND_HK);
    const int g_default = wide ? std::max(1, S / 8) : S;
    a.groups = std::max(1, std::min(std::min(p->groups > 0 ? p->groups : g_default, S), kMaxGroups));
    rc = alloc_large(ctx, G, S, tw);
    if (rc != GDE_OK) return rc;
    const size_t es = prec64 ? 8 : 4;
    const size_t slab = (size_t)S * n * es;
    // Interleaved FP32 solution slabs: when every query's {x, c} slab fits
    // in a third of the free memory, each query keeps its own slab (zeroed
    // here, in one pass) and its row is read out after the launch, so a
    // retiring slot only clears its residual.
    a.xq = 0;
    if (a.xld && x_out) {
        size_t freeb = 0, totb = 0;
        cudaMemGetInfo(&freeb, &totb);
        const size_t need = (size_t)nq * (size_t)a.xtile * 4;
        // under an HBM budget the query slabs count against it with the slots
        const bool in_budget = budget_bytes <= 0.0 ||
                               (double)S * (double)served_slot_bytes(n, G->g.cap, prec64, any_hk, base, G->g.hub_cut) +
                                       (double)need <= budget_bytes;
        if (need <= freeb / 3 && in_budget) {
            void* xq = wsget(ctx, "Xq", need);
            if (xq) {
                a.X = xq;
                a.XC = (float*)xq + 1;
                a.xq = 1;
            }
        }
    }
    // FP32 PPR / Katz slots: the residual of the highest-degree nodes in FP64
    a.RH = nullptr;
    a.rh_cut = 0;
    if (!prec64 && G->g.hub_cut > 0) {
        a.rh_cut = (int)std::min<int64_t>(G->g.hub_cut, kRhMax);
        a.RH = (double*)wsget(ctx, "RH", (size_t)S * a.rh_cut * 8);
        if (!a.RH) return fail(ctx, GDE_ENOMEM, "device memory exhausted (FP64 hub residuals)");
    }
    // Small queries (eps >= sparse_eps, PPR / Katz) go to hash-table blocks
    // when the launch writes per-query {x, c} slabs: their entries land in
    // the same slabs, so the read-out below serves both classes.
    std::vector<int32_t> ord_d, ord_s;
    int sp_cap = 0;
    if (p->sparse_blocks > 0 && p->sparse_eps > 0.0 && a.xq && !r_out) {
        for (int64_t q = 0; q < nq; q++) {
            const int k = kinds ? kinds[q] : kind;
            const bool small = (k == KIND_PPR || k == KIND_KATZ) && eps[q] >= p->sparse_eps;
            (small ? ord_s : ord_d).push_back((int32_t)q);
        }
        if (ord_s.empty()) ord_d.clear();
        sp_cap = 1024;
        while (sp_cap < (p->sparse_cap > 0 ? std::min(p->sparse_cap, 1 << 24) : (1 << 16))) sp_cap <<= 1;
    }
    const int spB = ord_s.empty() ? 0 : (int)std::min<int64_t>(p->sparse_blocks, (int64_t)ord_s.size());
    const int64_t nd = ord_s.empty() ? nq : (int64_t)ord_d.size();
    auto dq = [&](int64_t i) -> int64_t { return ord_s.empty() ? i : (int64_t)ord_d[i]; };
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    CK(cudaMemsetAsync(a.R, 0, slab, ctx->stream));
    if (a.RH) CK(cudaMemsetAsync(a.RH, 0, (size_t)S * a.rh_cut * 8, ctx->stream));
    if (a.xq) CK(cudaMemsetAsync(a.X, 0, (size_t)nq * (size_t)a.xtile * 4, ctx->stream));
    else CK(cudaMemsetAsync(a.X, 0, a.xld ? 2 * slab : slab, ctx->stream));  // interleaved: X and XC
    if (a.R2) CK(cudaMemsetAsync(a.R2, 0, slab, ctx->stream));
    if (a.XC && !a.xld) CK(cudaMemsetAsync(a.XC, 0, (size_t)S * n * 4, ctx->stream));
    // ---- the query queue on the device ----
    std::vector<int32_t> qs(nq), qk(nq), qnl(kinds ? nq : 0), qpo(kinds ? nq : 0);
    std::vector<double> qt(nq), qr0(nq), qal(nq);
    std::vector<long long> qarr(arrival_ms ? nq : 0);
    std::vector<double> psi_all;
    std::map<int64_t, int32_t> psi_at;
    for (int64_t q = 0; q < nq; q++) {
        const int k = kinds ? kinds[q] : kind;
        const double al = alphas ? alphas[q] : p->alpha;
        qk[q] = k;
        qal[q] = al;
        qs[q] = G->node_in(seeds[q]);
        if (k == KIND_PPR) qt[q] = eps[q] * al;              // eps * alpha * degree
        else if (k == KIND_KATZ) qt[q] = eps[q];             // eps * degree
        else qt[q] = std::exp(p->tau) * eps[q];              // e^tau * eps * degree / N / psi
        qr0[q] = (k == KIND_PPR) ? al : 1.0;
        if (k == KIND_HK) {
            const int64_t N = estimate_n(p->tau, .5 * eps[q]);  // hk_solver.py:216-218
            if (!psi_at.count(N)) {
                psi_at[N] = (int32_t)psi_all.size();
                std::vector<double> ps = psi_table(p->tau, N);
                psi_all.insert(psi_all.end(), ps.begin(), ps.end());
            }
            qnl[q] = (int32_t)N;
            qpo[q] = psi_at[N];
        }
        if (arrival_ms) qarr[q] = (long long)(arrival_ms[q] * 1e6);
    }
    auto dev = [&](const char* name, size_t bytes) { return wsget(ctx, name, std::max<size_t>(bytes, 8)); };
    int32_t* d_seed = (int32_t*)dev("q_seed", nq * 4);
    double* d_theta = (double*)dev("q_theta", nq * 8);
    double* d_r0 = (double*)dev("q_r0", nq * 8);
    long long* d_arr = arrival_ms ? (long long*)dev("q_arrival", nq * 8) : nullptr;
    double* d_oper = (double*)dev("q_oper", nq * 8);
    int* d_rounds = (int*)dev("q_rounds", nq * 4);
    unsigned long long* d_start = (unsigned long long*)dev("q_start", nq * 8);
    unsigned long long* d_finish = (unsigned long long*)dev("q_finish", nq * 8);
    int* d_next = (int*)dev("q_next", 4);
    if (!d_seed || !d_theta || !d_r0 || (arrival_ms && !d_arr) || !d_oper || !d_rounds || !d_start ||
        !d_finish || !d_next)
        return fail(ctx, GDE_ENOMEM, "query queue");
    CK(cudaMemcpyAsync(d_seed, qs.data(), nq * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_theta, qt.data(), nq * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_r0, qr0.data(), nq * 8, cudaMemcpyHostToDevice, ctx->stream));
    if (d_arr) CK(cudaMemcpyAsync(d_arr, qarr.data(), nq * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(d_start, 0, nq * 8, ctx->stream));
    CK(cudaMemsetAsync(d_finish, 0, nq * 8, ctx->stream));
    int32_t* d_kind = nullptr;
    double* d_alpha = nullptr;
    int32_t* d_nlev = nullptr;
    int32_t* d_poff = nullptr;
    double* d_psi = nullptr;
    if (kinds) {
        d_kind = (int32_t*)dev("q_kind", nq * 4);
        d_alpha = (double*)dev("q_alpha", nq * 8);
        d_nlev = (int32_t*)dev("q_nlev", nq * 4);
        d_poff = (int32_t*)dev("q_psioff", nq * 4);
        d_psi = (double*)dev("q_psi", std::max<size_t>(psi_all.size(), 1) * 8);
        if (!d_kind || !d_alpha || !d_nlev || !d_poff || !d_psi) return fail(ctx, GDE_ENOMEM, "query queue");
        CK(cudaMemcpyAsync(d_kind, qk.data(), nq * 4, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(d_alpha, qal.data(), nq * 8, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(d_nlev, qnl.data(), nq * 4, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(d_poff, qpo.data(), nq * 4, cudaMemcpyHostToDevice, ctx->stream));
        if (!psi_all.empty())
            CK(cudaMemcpyAsync(d_psi, psi_all.data(), psi_all.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    }
    // the leading queries that have arrived at launch start go straight into
    // slots; the other slots start idle and admit queries as they arrive
    int first = (int)std::min<int64_t>(S, nd);
    if (arrival_ms) {
        first = 0;
        while (first < S && first < nd && qarr[dq(first)] <= 0) first++;
    }
    CK(cudaMemcpyAsync(d_next, &first, 4, cudaMemcpyHostToDevice, ctx->stream));
    // ---- outputs: the caller's device rows, or staging rows copied back ----
    const size_t oes = out64 ? 8 : 4;
    void* dx = nullptr;
    void* dr = nullptr;
    // pinned host rows the device can address (cudaHostAlloc'd or registered):
    // per-query solution rows are written there directly after the launch,
    // with no staging buffer and no separate copy
    bool x_direct = false;
    if (x_out && out_mem != GDE_MEM_DEVICE && a.xq) {
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, x_out) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer) {
            dx = pa.devicePointer;
            x_direct = true;
        }
        cudaGetLastError();
    }
    if (x_out && !dx) dx = (out_mem == GDE_MEM_DEVICE) ? x_out : dev("serve_x", (size_t)nq * ld_out * oes);
    if (r_out) dr = (out_mem == GDE_MEM_DEVICE) ? r_out : dev("serve_r", (size_t)nq * ld_out * oes);
    if ((x_out && !dx) || (r_out && !dr)) return fail(ctx, GDE_ENOMEM, "output staging");
    // ---- the first S queries start in the slots ----
    std::vector<TileParams> tp(S);
    std::vector<TileState> ts(S);
    std::vector<ColState> cs(S);
    std::vector<InitCol> ic(first);
    for (int t = 0; t < S; t++) {
        TileParams& P = tp[t];
        memset(&P, 0, sizeof(P));
        const int64_t qi = (t < first) ? dq(t) : 0;  // the query slot t starts with
        const int k = (t < first) ? qk[qi] : kind;
        P.kind = k;
        P.method = (k == KIND_HK) ? M_HK_LOCAL : M_LOCAL_GD;
        P.ncols = 1;
        P.alpha = (t < first) ? qal[qi] : p->alpha;
        P.tau = p->tau;
        P.x_gain = 1.0;
        if (k == KIND_HK) {
            P.n_levels = qnl[qi];
            P.psi_tab = d_psi + qpo[qi];
        }
        TileState& T = ts[t];
        memset(&T, 0, sizeof(T));
        T.t0 = 0;
        T.stamp = ctx->stamp[t];
        ColState& C = cs[t];
        memset(&C, 0, sizeof(C));
        if (t >= first) {
            T.done = SLOT_IDLE;
            T.qid = -1;
            C.seed = -1;
            continue;
        }
        T.done = SLOT_LIVE;
        T.qid = (int)qi;
        C.live = 1;
        C.seed = qs[qi];
        C.theta = qt[qi];
        InitCol I{};
        I.tile = t;
        I.col = 0;
        I.seed = qs[qi];
        I.r0 = qr0[qi];
        ic[t] = I;
    }
    CK(cudaMemcpyAsync(a.tp, tp.data(), S * sizeof(TileParams), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(a.ts, ts.data(), S * sizeof(TileState), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(a.cs, cs.data(), S * sizeof(ColState), cudaMemcpyHostToDevice, ctx->stream));
    InitCol* d_ic = (InitCol*)dev("initcols", std::max(first, 1) * sizeof(InitCol));
    if (!d_ic) return fail(ctx, GDE_ENOMEM, "column tables");
    if (first > 0) {
        CK(cudaMemcpyAsync(d_ic, ic.data(), first * sizeof(InitCol), cudaMemcpyHostToDevice, ctx->stream));
        CK(init_columns(a, prec64, 1, d_ic, first, ctx->stream));
    }
    a.serve = 1;
    a.round_budget = 0x3fffffff;
    ServeQueue& Q = a.queue;
    Q.nq = (int)nq;
    Q.next = d_next;
    Q.seed = d_seed;
    Q.theta = d_theta;
    Q.r0 = d_r0;
    Q.arrival_ns = d_arr;
    Q.x_out = dx;
    Q.r_out = dr;
    Q.ld_out = ld_out;
    Q.out64 = out64;
    Q.seed_add = (kind == KIND_KATZ) ? -1.0 : 0.0;  // xt[s_node] -= 1. (katz_solver.py:243)
    Q.kind = d_kind;
    Q.alpha = d_alpha;
    Q.n_levels = d_nlev;
    Q.psi_off = d_poff;
    Q.psi = d_psi;
    Q.tau = p->tau;
    Q.hk_scale = std::exp(p->tau);
    Q.oper = d_oper;
    Q.rounds = d_rounds;
    Q.start_ns = d_start;
    Q.finish_ns = d_finish;
    Q.kind0 = kind;
    Q.alpha0 = p->alpha;
    if (spB > 0) {
        const int64_t ns = (int64_t)ord_s.size();
        int32_t* d_ord_d = (int32_t*)dev("q_order_d", ord_d.size() * 4);
        int32_t* d_ord_s = (int32_t*)dev("q_order_s", ns * 4);
        int* d_ovf = (int*)dev("sp_ovf", ns * 4);
        int* d_ctr = (int*)dev("sp_ctr", 4 * 4);  // next_s, ovf_cnt, ovf_next, sp_left
        const size_t ent = (size_t)spB * sp_cap;
        int32_t* d_keys = (int32_t*)dev("sp_keys", ent * 4);
        double* d_r = (double*)dev("sp_r", ent * 8);
        double* d_x = (double*)dev("sp_x", ent * 8);
        int32_t* d_list = (int32_t*)dev("sp_list", ent * 3 * 4);
        double* d_push = (double*)dev("sp_push", ent * 8);
        if (!d_ord_d || !d_ord_s || !d_ovf || !d_ctr || !d_keys || !d_r || !d_x || !d_list || !d_push)
            return fail(ctx, GDE_ENOMEM, "small-query tables");
        if (!ord_d.empty())
            CK(cudaMemcpyAsync(d_ord_d, ord_d.data(), ord_d.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(d_ord_s, ord_s.data(), ns * 4, cudaMemcpyHostToDevice, ctx->stream));
        const int ctr[4] = {0, 0, 0, (int)ns};
        CK(cudaMemcpyAsync(d_ctr, ctr, sizeof ctr, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemsetAsync(d_ovf, 0xff, ns * 4, ctx->stream));
        CK(cudaMemsetAsync(d_keys, 0xff, ent * 4, ctx->stream));  // -1: empty
        CK(cudaMemsetAsync(d_r, 0, ent * 8, ctx->stream));
        CK(cudaMemsetAsync(d_x, 0, ent * 8, ctx->stream));
        Q.sp_blocks = spB;
        Q.sp_cap = sp_cap;
        Q.order_d = d_ord_d;
        Q.nd = (int)ord_d.size();
        Q.order_s = d_ord_s;
        Q.ns = (int)ns;
        Q.next_s = d_ctr;
        Q.ovf_cnt = d_ctr + 1;
        Q.ovf_next = d_ctr + 2;
        Q.sp_left = d_ctr + 3;
        Q.ovf = d_ovf;
        Q.sp_keys = d_keys;
        Q.sp_r = d_r;
        Q.sp_x = d_x;
        Q.sp_list = d_list;
        Q.sp_push = d_push;
    }
    double kernel_ms = 0.0;
    rc = run_engine(ctx, a, prec64, 1, stats, &kernel_ms);
    if (rc != GDE_OK) return rc;
    // ---- results ----
    // per-query solution slabs: every solution row at once, in caller order
    if (a.xq)
        CK(query_rows((const float*)a.X, a.xtile, G->perm_d, x_direct ? nullptr : G->iperm_d, n, nq, d_seed, d_kind,
                      Q.seed_add, Q.hk_scale, dx, out64, ld_out, ctx->stream));
    // retired rows are in internal node order: permute them to caller order
    // through a wave buffer of a few rows (random reads stay in L2)
    if (G->perm_d) {
        const int64_t row_bytes = n * (int64_t)oes;
        const int64_t wave = std::max<int64_t>(1, std::min<int64_t>(nq, (int64_t)(48 << 20) / row_bytes));
        void* tmp = dev("out_wave", (size_t)(wave * row_bytes));
        if (!tmp) return fail(ctx, GDE_ENOMEM, "output permutation buffer");
        for (void* rows : {a.xq ? nullptr : dx, dr}) {
            if (!rows) continue;
            for (int64_t q0 = 0; q0 < nq; q0 += wave) {
                const int64_t w = std::min<int64_t>(wave, nq - q0);
                char* at = (char*)rows + (size_t)q0 * ld_out * oes;
                CK(cudaMemcpy2DAsync(tmp, row_bytes, at, ld_out * oes, row_bytes, w, cudaMemcpyDeviceToDevice,
                                     ctx->stream));
                CK(permute_entries(tmp, n, at, ld_out, G->perm_d, n, w, (int)oes, ctx->stream));
            }
        }
    }
    if (out_mem != GDE_MEM_DEVICE) {
        if (x_out && !x_direct)
            CK(cudaMemcpyAsync(x_out, dx, (size_t)nq * ld_out * oes, cudaMemcpyDeviceToHost, ctx->stream));
        if (r_out) CK(cudaMemcpyAsync(r_out, dr, (size_t)nq * ld_out * oes, cudaMemcpyDeviceToHost, ctx->stream));
    }
    std::vector<double> hop(nq);
    std::vector<int> hro(nq);
    std::vector<unsigned long long> hst(nq), hfi(nq);
    CK(cudaMemcpyAsync(hop.data(), d_oper, nq * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(hro.data(), d_rounds, nq * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(hst.data(), d_start, nq * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(hfi.data(), d_finish, nq * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(ctx->hts, a.ts, S * sizeof(TileState), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const unsigned long long k0 = ctx->hstats->start_ns;
    bool capped = false;
    for (int t = 0; t < S; t++) {
        const TileState& T = ctx->hts[t];
        ctx->stamp[t] = T.stamp + (int)std::max<long long>(0, (long long)ctx->hstats->iters - T.t0) + 4;
        if (T.done == SLOT_LIVE) capped = true;
    }
    for (int64_t q = 0; q < nq; q++) {
        if (oper_out) oper_out[q] = hop[q];
        if (rounds_out) rounds_out[q] = hro[q];
        if (lat_ms_out) {
            // from arrival (served) or admission (first slots: the launch start)
            unsigned long long from = arrival_ms ? k0 + (unsigned long long)qarr[q] : (hst[q] ? hst[q] : k0);
            lat_ms_out[q] = hfi[q] > from ? (float)((double)(hfi[q] - from) * 1e-6) : 0.f;
        }
    }
    if (stats) {
        float tot = 0.f;
        cudaEventElapsedTime(&tot, ctx->ev[2], ctx->ev[3]);
        stats->total_ms = tot;
        stats->kernel_ms = kernel_ms;
        stats->tiles = S;
        stats->tile_w = 1;
    }
    if (capped) return fail(ctx, GDE_EITERCAP, "max_rounds reached before the stopping rule held");
    return GDE_OK;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* gde_status_str(int s) {
    switch (s) {
        case GDE_OK: return "ok";
        case GDE_EINVAL: return "invalid argument";
        case GDE_ENOMEM: return "out of memory";
        case GDE_EITERCAP: return "round cap reached";
        case GDE_ECUDA: return "CUDA error";
        case GDE_EHANG: return "device-side wait ran out";
        case GDE_ECAPACITY: return "padded row out of slack";
        case GDE_ENOTFOUND: return "not found";
    }
    return "unknown status";
}

int gde_version(void) { return 1; }

int gde_ctx_create(int device, gde_ctx** out) {
    if (!out) return GDE_EINVAL;
    *out = nullptr;
    gde_ctx* ctx = new gde_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete ctx; return GDE_ECUDA; }
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
    cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    if (!coop) { delete ctx; return GDE_ECUDA; }
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ctx->bar, kMaxGroups * sizeof(GridBarrier)) != cudaSuccess ||
        cudaMalloc(&ctx->derr, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&ctx->dstats, sizeof(LaunchStats)) != cudaSuccess ||
        cudaMallocHost(&ctx->hstats, sizeof(LaunchStats)) != cudaSuccess ||
        cudaMallocHost(&ctx->hts, sizeof(TileState) * 4096) != cudaSuccess) {
        delete ctx;
        return GDE_ECUDA;
    }
    for (auto& ev : ctx->ev) cudaEventCreate(&ev);
    *out = ctx;
    return GDE_OK;
}

int gde_ctx_destroy(gde_ctx* ctx) {
    if (!ctx) return GDE_EINVAL;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ws_release_all(ctx);
    if (ctx->plain_n >= 0) {
        cudaFree(ctx->plain.xt); cudaFree(ctx->plain.rt); cudaFree(ctx->plain.tmp); cudaFree(ctx->plain.sp);
        cudaFree(ctx->plain.eps_vec); cudaFree(ctx->plain.queue); cudaFree(ctx->plain.nz);
        cudaFree(ctx->plain.d_count); cudaFree(ctx->plain.d_oper); cudaFreeHost(ctx->plain.h_count);
    }
    if (ctx->trace) cudaFree(ctx->trace);
    cudaFree(ctx->bar);
    cudaFree(ctx->derr);
    cudaFree(ctx->dstats);
    cudaFreeHost(ctx->hstats);
    cudaFreeHost(ctx->hts);
    for (auto& ev : ctx->ev) cudaEventDestroy(ev);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GDE_OK;
}

const char* gde_last_error(gde_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

void* gde_ctx_stream(gde_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int gde_ctx_trace(gde_ctx* ctx, int iters) {
    if (!ctx || iters < 0) return fail(ctx, GDE_EINVAL, "bad trace arguments");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->trace) cudaFree(ctx->trace);
    ctx->trace = nullptr;
    ctx->trace_iters = 0;
    ctx->trace_grid = 0;
    if (iters == 0) return GDE_OK;
    // room for the largest co-resident grid of any push-kernel instantiation
    const size_t bytes = (size_t)iters * ctx->sms * 32 * kTracePoints * 8;
    if (cudaMalloc(&ctx->trace, bytes) != cudaSuccess) {
        cudaGetLastError();
        ctx->trace = nullptr;
        return fail(ctx, GDE_ENOMEM, "trace buffer");
    }
    CK(cudaMemsetAsync(ctx->trace, 0, bytes, ctx->stream));
    ctx->trace_iters = iters;
    return GDE_OK;
}

int gde_ctx_set_wait_limit(gde_ctx* ctx, int64_t polls) {
    if (!ctx || polls < 0) return fail(ctx, GDE_EINVAL, "bad wait limit");
    ctx->wait_limit = polls;
    return GDE_OK;
}

int gde_ctx_trace_read(gde_ctx* ctx, uint64_t* out, int64_t cap, int* iters, int* grid, int* points) {
    if (!ctx) return GDE_EINVAL;
    if (iters) *iters = ctx->trace_iters;
    if (grid) *grid = ctx->trace_grid;
    if (points) *points = kTracePoints;
    if (!ctx->trace || !out) return GDE_OK;
    const int64_t need = (int64_t)ctx->trace_iters * ctx->trace_grid * kTracePoints;
    if (cap < need) return fail(ctx, GDE_EINVAL, "trace output too small");
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(out, ctx->trace, (size_t)need * 8, cudaMemcpyDeviceToHost));
    return GDE_OK;
}

int gde_serve(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t nq, const int32_t* seeds, const double* eps,
              const double* arrival_ms, void* x_out, void* r_out, int out64, int out_mem, int64_t ld_out,
              double* oper_out, int32_t* rounds_out, float* lat_ms_out, gde_stats* stats) {
    if (!ctx || !G || !p || nq < 0 || (nq > 0 && (!seeds || !eps))) return fail(ctx, GDE_EINVAL, "bad serve arguments");
    if (p->method != M_LOCAL_GD || (p->kind != KIND_PPR && p->kind != KIND_KATZ))
        return fail(ctx, GDE_EINVAL, "served queries are PPR or Katz local GD");
    CK(cudaSetDevice(ctx->device));
    const int64_t n = G->g.n;
    if (ld_out < n && (x_out || r_out)) return fail(ctx, GDE_EINVAL, "ld_out < n");
    for (int64_t q = 0; q < nq; q++) {
        if (seeds[q] < 0 || seeds[q] >= n) return fail(ctx, GDE_EINVAL, "seed out of range");
        if (!(eps[q] > 0.0)) return fail(ctx, GDE_EINVAL, "eps must be > 0");
        if (arrival_ms && !(arrival_ms[q] >= 0.0)) return fail(ctx, GDE_EINVAL, "arrival times must be >= 0");
        if (arrival_ms && q > 0 && arrival_ms[q] < arrival_ms[q - 1])
            return fail(ctx, GDE_EINVAL, "arrival times must be non-decreasing (queries are admitted in order)");
        if (p->kind == KIND_PPR && !(eps[q] * G->h_deg[G->node_in(seeds[q])] <= 1.))
            return fail(ctx, GDE_EINVAL, "eps * degree[s_node] > 1 (ppr_solver.py:213)");
    }
    if (stats) memset(stats, 0, sizeof(*stats));
    if (nq == 0) return GDE_OK;
    gde_params pp = *p;
    pp.prec = katz_compute_prec(ctx, G, p);
    p = &pp;
    if (stats) stats->prec = p->prec;
    return solve_served(ctx, G, p, nq, seeds, eps, arrival_ms, x_out, r_out, out64, out_mem, ld_out, oper_out,
                        rounds_out, lat_ms_out, stats);
}

int gde_serve_mixed(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t nq, const int32_t* kinds,
                    const int32_t* seeds, const double* eps, const double* alphas, const double* arrival_ms,
                    double hbm_budget_bytes, void* x_out, int out64, int out_mem, int64_t ld_out, double* oper_out,
                    int32_t* rounds_out, float* lat_ms_out, gde_stats* stats) {
    if (!ctx || !G || !p || nq < 0 || (nq > 0 && (!seeds || !eps || !kinds)))
        return fail(ctx, GDE_EINVAL, "bad serve arguments");
    CK(cudaSetDevice(ctx->device));
    const int64_t n = G->g.n;
    if (ld_out < n && x_out) return fail(ctx, GDE_EINVAL, "ld_out < n");
    bool any_hk = false;
    for (int64_t q = 0; q < nq; q++) {
        const int k = kinds[q];
        if (k != KIND_PPR && k != KIND_KATZ && k != KIND_HK)
            return fail(ctx, GDE_EINVAL, "query kinds are GDE_PPR, GDE_KATZ or GDE_HK");
        any_hk |= (k == KIND_HK);
        if (seeds[q] < 0 || seeds[q] >= n) return fail(ctx, GDE_EINVAL, "seed out of range");
        if (!(eps[q] > 0.0)) return fail(ctx, GDE_EINVAL, "eps must be > 0");
        if (arrival_ms && !(arrival_ms[q] >= 0.0)) return fail(ctx, GDE_EINVAL, "arrival times must be >= 0");
        if (arrival_ms && q > 0 && arrival_ms[q] < arrival_ms[q - 1])
            return fail(ctx, GDE_EINVAL, "arrival times must be non-decreasing (queries are admitted in order)");
        const double al = alphas ? alphas[q] : p->alpha;
        if (k != KIND_HK && !(al > 0.0)) return fail(ctx, GDE_EINVAL, "alpha must be > 0");
        if (k == KIND_PPR && !(eps[q] * G->h_deg[G->node_in(seeds[q])] <= 1.))
            return fail(ctx, GDE_EINVAL, "eps * degree[s_node] > 1 (ppr_solver.py:213)");
    }
    if (any_hk && !(p->tau >= 1.0)) return fail(ctx, GDE_EINVAL, "tau must be >= 1 (hk_solver.py:35)");
    if (stats) memset(stats, 0, sizeof(*stats));
    if (nq == 0) return GDE_OK;
    gde_params pp = *p;
    pp.method = M_LOCAL_GD;
    pp.kind = kinds[0] == KIND_HK ? KIND_PPR : kinds[0];
    return solve_served(ctx, G, &pp, nq, seeds, eps, arrival_ms, x_out, nullptr, out64, out_mem, ld_out, oper_out,
                        rounds_out, lat_ms_out, stats, kinds, alphas, hbm_budget_bytes);
}

int gde_ctx_sync(gde_ctx* ctx) {
    if (!ctx) return GDE_EINVAL;
    CK(cudaStreamSynchronize(ctx->stream));
    return GDE_OK;
}

int64_t gde_hk_estimate_n(double tau, double eps) {
    if (!(tau >= 1.0) || !(eps > 0.0)) return -1;  // hk_solver.py:35-36
    return estimate_n(tau, eps);
}

int gde_graph_upload(gde_ctx* ctx, int64_t n, int64_t cap, const int64_t* indptr, const int32_t* indices,
                     const int64_t* row_len, const double* degree, gde_graph** out) {
    if (!ctx || !out || n <= 0 || !indptr || !indices || cap < 0) return fail(ctx, GDE_EINVAL, "bad graph arguments");
    if (n >= (int64_t)1 << 31) return fail(ctx, GDE_EINVAL, "node ids must fit in int32");
    *out = nullptr;
    CK(cudaSetDevice(ctx->device));
    gde_graph* G = new gde_graph();
    G->ctx = ctx;
    std::vector<int64_t> len0(n);
    std::vector<double> deg0(n);
    for (int64_t u = 0; u < n; u++) {
        int64_t len = row_len ? row_len[u] : indptr[u + 1] - indptr[u];
        if (len < 0 || indptr[u] + len > cap || indptr[u] + len > indptr[u + 1]) {
            delete G;
            return fail(ctx, GDE_EINVAL, "row " + std::to_string(u) + " exceeds its CSR extent");
        }
        len0[u] = len;
        deg0[u] = degree ? degree[u] : (double)len;
        if (degree && degree[u] != (double)len) G->deg_is_len = false;
    }
    for (int64_t j = 0; j < cap; j++)
        if (indices[j] < 0 || indices[j] >= n) {
            // slack slots of a padded CSR may hold the sentinel n
            if (row_len && indices[j] == n) continue;
            delete G;
            return fail(ctx, GDE_EINVAL, "column index out of range at position " + std::to_string(j));
        }
    if (row_len)  // ... but a row's live entries are node ids
        for (int64_t u = 0; u < n; u++)
            for (int64_t j = indptr[u]; j < indptr[u] + len0[u]; j++)
                if (indices[j] == n) {
                    delete G;
                    return fail(ctx, GDE_EINVAL, "row " + std::to_string(u) + " holds the padding sentinel at "
                                "position " + std::to_string(j) + ", inside its row length");
                }
    std::vector<int32_t> col_new;
    const int32_t* col_src = indices;
    int64_t cap_new = cap;
    if (!row_len) {
        // static CSR: relabel by descending degree (stable), rows sorted
        G->relabeled = true;
        std::vector<int32_t> iperm(n);
        for (int64_t u = 0; u < n; u++) iperm[u] = (int32_t)u;
        std::stable_sort(iperm.begin(), iperm.end(), [&](int32_t a, int32_t b) { return len0[a] > len0[b]; });
        G->h_perm.resize(n);
        for (int64_t k = 0; k < n; k++) G->h_perm[iperm[k]] = (int32_t)k;
        G->h_indptr.assign(n + 1, 0);
        G->h_len.resize(n);
        G->h_deg.resize(n);
        for (int64_t k = 0; k < n; k++) {
            G->h_len[k] = len0[iperm[k]];
            G->h_deg[k] = deg0[iperm[k]];
            G->h_indptr[k + 1] = G->h_indptr[k] + G->h_len[k];
        }
        cap_new = G->h_indptr[n];
        col_new.resize(std::max<int64_t>(cap_new, 1));
        for (int64_t k = 0; k < n; k++) {
            const int64_t src = indptr[iperm[k]], dst = G->h_indptr[k];
            for (int64_t j = 0; j < G->h_len[k]; j++) col_new[dst + j] = G->h_perm[indices[src + j]];
            std::sort(col_new.begin() + dst, col_new.begin() + dst + G->h_len[k]);
        }
        col_src = col_new.data();
    } else {
        G->h_indptr.assign(indptr, indptr + n + 1);
        G->h_len = len0;
        G->h_deg = deg0;
    }
    cap = cap_new;
    G->g.n = n;
    G->g.cap = cap;
    // row_ptr gets two spare entries so aligned 16-byte windows stay in bounds
    cudaError_t e = cudaMalloc(&G->row_ptr, (n + 3) * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&G->col, std::max<int64_t>(cap, 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&G->row_len, n * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&G->degf, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&G->degd, n * sizeof(double));
    if (e != cudaSuccess) {
        cudaFree(G->row_ptr); cudaFree(G->col); cudaFree(G->row_len); cudaFree(G->degf); cudaFree(G->degd);
        delete G;
        return fail(ctx, GDE_ENOMEM, "device memory exhausted (graph)");
    }
    CK(cudaMemsetAsync(G->row_ptr, 0, (n + 3) * sizeof(int64_t), ctx->stream));
    CK(cudaMemcpyAsync(G->row_ptr, G->h_indptr.data(), (n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                       ctx->stream));
    if (cap > 0) CK(cudaMemcpyAsync(G->col, col_src, cap * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    if (G->relabeled) {
        CK(cudaMalloc(&G->perm_d, n * sizeof(int32_t)));
        CK(cudaMemcpyAsync(G->perm_d, G->h_perm.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
        std::vector<int32_t> inv(n);
        for (int64_t u = 0; u < n; u++) inv[G->h_perm[u]] = (int32_t)u;
        CK(cudaMalloc(&G->iperm_d, n * sizeof(int32_t)));
        CK(cudaMemcpyAsync(G->iperm_d, inv.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));  // inv is released on return
    }
    G->g.perm = G->perm_d;
    // hubs: the degree-sorted prefix of nodes with more than 64 neighbours;
    // pushes into them are combined per warp before the atomic
    G->g.hub_cut = 0;
    if (G->relabeled)
        while (G->g.hub_cut < n && G->h_len[G->g.hub_cut] > kHubLen) G->g.hub_cut++;
    G->g.row_ptr = G->row_ptr;
    G->g.col = G->col;
    G->g.row_len = G->row_len;
    G->g.degf = G->degf;
    G->g.degd = G->degd;
    int rc = upload_degrees(ctx, G);
    if (rc != GDE_OK) { gde_graph_free(G); return rc; }
    if (G->relabeled) {
        rc = build_static_records(ctx, G, col_src);
        if (rc != GDE_OK) { gde_graph_free(G); return rc; }
    }
    *out = G;
    return GDE_OK;
}

int gde_graph_free(gde_graph* G) {
    if (!G) return GDE_EINVAL;
    cudaSetDevice(G->ctx->device);
    cudaStreamSynchronize(G->ctx->stream);
    cudaFree(G->row_ptr); cudaFree(G->col); cudaFree(G->row_len); cudaFree(G->degf); cudaFree(G->degd);
    cudaFree(G->nfac); cudaFree(G->tfac); cudaFree(G->tfac_f); cudaFree(G->perm_d); cudaFree(G->iperm_d);
    cudaFree(G->col_deg); cudaFree(G->rec);
    cudaFree(G->pw1); cudaFree(G->pwb);
    delete G;
    return GDE_OK;
}

int gde_graph_info(gde_graph* G, int64_t* n, int64_t* cap, double* vol) {
    if (!G) return GDE_EINVAL;
    if (n) *n = G->g.n;
    if (cap) *cap = G->g.cap;
    if (vol) *vol = G->g.vol;
    return GDE_OK;
}

int gde_solve(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t nq, const int32_t* seeds, const double* eps,
              void* x_out, void* r_out, int out64, int out_mem, int64_t ld_out, double* oper_out, int32_t* rounds_out,
              float* lat_ms_out, gde_stats* stats) {
    if (!ctx || !G || !p || nq < 0 || (nq > 0 && (!seeds || !eps))) return fail(ctx, GDE_EINVAL, "bad solve arguments");
    CK(cudaSetDevice(ctx->device));
    const int64_t n = G->g.n;
    const int kind = p->kind, method = p->method;
    if (kind != KIND_PPR && kind != KIND_KATZ && kind != KIND_HK) return fail(ctx, GDE_EINVAL, "kind must be PPR, KATZ or HK");
    const bool hk = method_is_hk(method);
    if (hk != (kind == KIND_HK)) return fail(ctx, GDE_EINVAL, "heat-kernel methods go with GDE_HK only");
    if (method < M_LOCAL_GD || method > M_HK_TAYLOR) return fail(ctx, GDE_EINVAL, "unknown method");
    if (ld_out < n && (x_out || r_out)) return fail(ctx, GDE_EINVAL, "ld_out < n");
    for (int64_t q = 0; q < nq; q++) {
        if (seeds[q] < 0 || seeds[q] >= n) return fail(ctx, GDE_EINVAL, "seed out of range");
        if (!(eps[q] > 0.0)) return fail(ctx, GDE_EINVAL, "eps must be > 0");
        if (kind == KIND_PPR && (method == M_LOCAL_GD || method == M_GLOBAL_GD) && !(eps[q] * G->h_deg[G->node_in(seeds[q])] <= 1.))
            return fail(ctx, GDE_EINVAL, "eps * degree[s_node] > 1 (ppr_solver.py:213)");
    }
    if (hk && !(p->tau >= 1.0)) return fail(ctx, GDE_EINVAL, "tau must be >= 1 (hk_solver.py:35)");
    // HK relaxation: 0 or 1 is none; the relaxed push converges for 0 < omega < 2
    const bool relax = (method == M_HK_LOCAL || method == M_HK_GLOBAL) && p->omega != 0.0 && p->omega != 1.0;
    if (relax && !(p->omega > 0.0 && p->omega < 2.0)) return fail(ctx, GDE_EINVAL, "HK omega must be in (0, 2)");
    if (relax && p->prec != GDE_FP64) return fail(ctx, GDE_EINVAL, "HK relaxation omega != 1 runs in FP64");
    if (stats) memset(stats, 0, sizeof(*stats));
    if (nq == 0) return GDE_OK;
    gde_params pp = *p;
    pp.prec = katz_compute_prec(ctx, G, p);
    p = &pp;
    if (stats) stats->prec = p->prec;
    const int prec64 = (p->prec == GDE_FP64);

    // PPR / Katz local GD with one column per tile runs as a served queue:
    // slots cycle through the queries inside one persistent launch.
    const bool crossing = (method == M_LOCAL_GD) && (kind == KIND_PPR || kind == KIND_KATZ);
    if (crossing && p->tile_w <= 1)
        return solve_served(ctx, G, p, nq, seeds, eps, nullptr, x_out, r_out, out64, out_mem, ld_out, oper_out,
                            rounds_out, lat_ms_out, stats);

    int W = p->tile_w;
    if (W <= 0) W = (nq == 1) ? 1 : (prec64 ? 4 : 8);
    while (W > 1 && W > nq * 2) W >>= 1;
    if (!valid_w(W)) return fail(ctx, GDE_EINVAL, "tile_w must be 1, 2, 4, 8, 16 or 32");

    // Group queries into tiles.  HK tiles never mix Taylor lengths.
    std::vector<int64_t> order(nq);
    for (int64_t q = 0; q < nq; q++) order[q] = q;
    std::vector<int64_t> Nq(nq, 0);
    if (hk) {
        for (int64_t q = 0; q < nq; q++)
            Nq[q] = (method == M_HK_TAYLOR) ? estimate_n(p->tau, eps[q]) : estimate_n(p->tau, .5 * eps[q]);
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return Nq[a] < Nq[b]; });
    }
    struct TileDef { std::vector<int64_t> qs; int64_t N; };
    std::vector<TileDef> tiles;
    for (int64_t i = 0; i < nq;) {
        TileDef td;
        td.N = Nq[order[i]];
        while (i < nq && (int)td.qs.size() < W && Nq[order[i]] == td.N) td.qs.push_back(order[i++]);
        tiles.push_back(td);
    }

    // Memory per tile; launch groups sized to the free device memory.
    const size_t es = prec64 ? 8 : 4;
    size_t per_tile = (size_t)n * W * es * (3 + (hk ? 1 : 0) + (method_is_cheby(method) ? 1 : 0)) +
                      (size_t)n * W * (prec64 ? 0 : 4) + (size_t)n * 4 * 6 + 4096;
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    size_t have = 0;
    for (auto& kv : ctx->ws) have += kv.second.bytes;
    size_t budget = (size_t)((double)(freeb + have) * 0.85);
    int max_tiles = (int)std::min<size_t>(512, std::max<size_t>(1, budget / std::max<size_t>(per_tile, 1)));

    PushArgs base{};
    fill_tuning(p, base);
    const double m_vol = G->g.vol;
    double kernel_ms = 0.0;
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));

    // per-launch tables
    std::vector<double> ctab;
    if (method_is_cheby(method)) ctab = cheby_table(kind, p->alpha, p->l_max, p->mu_min, base.max_rounds + 2);
    std::map<int64_t, std::vector<double>> psis;
    if (hk)
        for (auto& td : tiles)
            if (!psis.count(td.N)) {
                if (method == M_HK_TAYLOR) psis[td.N] = std::vector<double>(td.N + 2, 1.0);
                else psis[td.N] = psi_table(p->tau, td.N);
            }
    double* d_ctab = nullptr;
    if (!ctab.empty()) {
        d_ctab = (double*)wsget(ctx, "ctab", ctab.size() * 8);
        if (!d_ctab) return fail(ctx, GDE_ENOMEM, "coefficient table");
        CK(cudaMemcpyAsync(d_ctab, ctab.data(), ctab.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    }
    std::map<int64_t, double*> d_psi;
    if (hk) {
        size_t tot = 0;
        for (auto& kv : psis) tot += kv.second.size();
        double* buf = (double*)wsget(ctx, "psi", tot * 8);
        if (!buf) return fail(ctx, GDE_ENOMEM, "psi table");
        size_t off = 0;
        for (auto& kv : psis) {
            CK(cudaMemcpyAsync(buf + off, kv.second.data(), kv.second.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
            d_psi[kv.first] = buf + off;
            off += kv.second.size();
        }
    }

    for (size_t t0 = 0; t0 < tiles.size(); t0 += max_tiles) {
        const int nt = (int)std::min<size_t>(max_tiles, tiles.size() - t0);
        TileWs tw;
        tw.a = base;
        int rc = alloc_tiles(ctx, G, nt, W, prec64, hk, method_is_cheby(method), true, !prec64, tw);
        if (rc != GDE_OK) return rc;
        PushArgs& a = tw.a;
        a.small_max = base.small_max; a.med_max = base.med_max; a.chunk = base.chunk;
        a.dense_div = base.dense_div; a.max_rounds = base.max_rounds; a.allow_dense = base.allow_dense;
        rc = alloc_large(ctx, G, nt, tw);
        if (rc != GDE_OK) return rc;
        const size_t slab = (size_t)nt * n * W * es;
        CK(cudaMemsetAsync(a.R, 0, slab, ctx->stream));
        CK(cudaMemsetAsync(a.X, 0, a.xld ? 2 * slab : slab, ctx->stream));  // interleaved: X and XC
        if (a.R2) CK(cudaMemsetAsync(a.R2, 0, slab, ctx->stream));
        if (a.DX) CK(cudaMemsetAsync(a.DX, 0, slab, ctx->stream));
        if (a.XC && !a.xld) CK(cudaMemsetAsync(a.XC, 0, (size_t)nt * n * W * 4, ctx->stream));
        std::vector<TileParams> tp(nt);
        std::vector<TileState> ts(nt);
        std::vector<ColState> cs((size_t)nt * W);
        std::vector<InitCol> ic;
        std::vector<ExtractCol> ec;
        for (int t = 0; t < nt; t++) {
            const TileDef& td = tiles[t0 + t];
            TileParams& P = tp[t];
            memset(&P, 0, sizeof(P));
            P.kind = kind;
            P.method = method;
            P.ncols = (int)td.qs.size();
            P.n_levels = (int)td.N;
            P.alpha = p->alpha;
            P.tau = p->tau;
            P.l_max = p->l_max;
            P.mu_min = p->mu_min;
            P.x_gain = 1.0;
            P.coef_tab = d_ctab;
            P.psi_tab = hk ? d_psi[td.N] : nullptr;
            P.omega = relax ? p->omega : 0.0;
            TileState& S = ts[t];
            memset(&S, 0, sizeof(S));
            S.dense_next[0] = method_is_global(method) ? 1 : 0;
            S.stamp = ctx->stamp[t];
            for (int c = 0; c < W; c++) {
                ColState& C = cs[(size_t)t * W + c];
                memset(&C, 0, sizeof(C));
                C.seed = -1;
                if (c >= P.ncols) continue;
                int64_t q = td.qs[c];
                C.live = 1;
                C.seed = G->node_in(seeds[q]);
                if (kind == KIND_PPR) C.theta = eps[q] * p->alpha;      // eps * alpha * degree
                else if (kind == KIND_KATZ) C.theta = eps[q];            // eps * degree
                else C.theta = std::exp(p->tau) * eps[q];                // np.exp(tau) * eps * degree / est_n
                InitCol I{};
                I.tile = t;
                I.col = c;
                I.seed = G->node_in(seeds[q]);
                const double ds = G->h_deg[I.seed];
                if (method_is_cheby(method)) {
                    if (kind == KIND_KATZ) {
                        I.x0 = 2. / (p->l_max + p->mu_min);
                        I.dx0 = I.x0;
                        I.r0 = 1. - 2. / (p->l_max + p->mu_min);
                        I.push0 = 2. * p->alpha / (p->l_max + p->mu_min);
                    } else {
                        I.x0 = p->alpha;
                        I.dx0 = p->alpha;
                        I.r0 = 0.0;
                        I.push0 = (1. - p->alpha) * p->alpha / ds;
                    }
                } else {
                    I.r0 = (kind == KIND_PPR) ? p->alpha : 1.0;
                }
                ic.push_back(I);
                ExtractCol E{};
                E.tile = t;
                E.col = c;
                E.out_row = q;
                E.seed = (kind == KIND_KATZ && (method == M_LOCAL_GD || method == M_GLOBAL_GD)) ? seeds[q] : -1;
                E.seed_add = -1.0;  // xt[s_node] -= 1. (katz_solver.py:243)
                E.scale = hk ? std::exp(p->tau) : 1.0;  // xt /= np.exp(tau)
                E.r_levels = (hk && method != M_HK_TAYLOR) ? 2 : 1;
                ec.push_back(E);
            }
        }
        CK(cudaMemcpyAsync(a.tp, tp.data(), nt * sizeof(TileParams), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(a.ts, ts.data(), nt * sizeof(TileState), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(a.cs, cs.data(), cs.size() * sizeof(ColState), cudaMemcpyHostToDevice, ctx->stream));
        InitCol* d_ic = (InitCol*)wsget(ctx, "initcols", ic.size() * sizeof(InitCol));
        ExtractCol* d_ec = (ExtractCol*)wsget(ctx, "extcols", ec.size() * sizeof(ExtractCol));
        if (!d_ic || !d_ec) return fail(ctx, GDE_ENOMEM, "column tables");
        CK(cudaMemcpyAsync(d_ic, ic.data(), ic.size() * sizeof(InitCol), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(d_ec, ec.data(), ec.size() * sizeof(ExtractCol), cudaMemcpyHostToDevice, ctx->stream));
        CK(init_columns(a, prec64, W, d_ic, (int)ic.size(), ctx->stream));
        rc = run_engine(ctx, a, prec64, W, stats, &kernel_ms);
        if (rc != GDE_OK) return rc;
        // results
        const size_t oes = out64 ? 8 : 4;
        const int rl = (hk && method != M_HK_TAYLOR) ? 2 : 1;
        if (out_mem == GDE_MEM_DEVICE) {
            CK(extract_columns(a, prec64, W, d_ec, (int)ec.size(), x_out, r_out, out64, ld_out, n, 0, ctx->stream));
        } else if (x_out || r_out) {
            // stage through device memory in chunks of columns
            size_t row_b = (size_t)ld_out * oes;
            int64_t per = std::max<int64_t>(1, (int64_t)((size_t)512 << 20) / (int64_t)(row_b * (1 + rl)));
            for (size_t e0 = 0; e0 < ec.size(); e0 += per) {
                size_t ne = std::min<size_t>(per, ec.size() - e0);
                std::vector<ExtractCol> sub(ec.begin() + e0, ec.begin() + e0 + ne);
                for (size_t i = 0; i < ne; i++) sub[i].out_row = (int64_t)i;
                ExtractCol* d_sub = (ExtractCol*)wsget(ctx, "extsub", ne * sizeof(ExtractCol));
                void* sx = x_out ? wsget(ctx, "stage_x", ne * row_b) : nullptr;
                void* sr = r_out ? wsget(ctx, "stage_r", ne * row_b * rl) : nullptr;
                if (!d_sub || (x_out && !sx) || (r_out && !sr)) return fail(ctx, GDE_ENOMEM, "staging buffers");
                CK(cudaMemcpyAsync(d_sub, sub.data(), ne * sizeof(ExtractCol), cudaMemcpyHostToDevice, ctx->stream));
                CK(extract_columns(a, prec64, W, d_sub, (int)ne, sx, sr, out64, ld_out, n, 0, ctx->stream));
                for (size_t i = 0; i < ne; i++) {
                    int64_t q = ec[e0 + i].out_row;
                    if (x_out)
                        CK(cudaMemcpyAsync((char*)x_out + q * row_b, (char*)sx + i * row_b, row_b,
                                           cudaMemcpyDeviceToHost, ctx->stream));
                    if (r_out)
                        CK(cudaMemcpyAsync((char*)r_out + q * row_b * rl, (char*)sr + i * row_b * rl, row_b * rl,
                                           cudaMemcpyDeviceToHost, ctx->stream));
                }
            }
        }
        // per-column counters and stamp bookkeeping
        std::vector<ColState> hcs(cs.size());
        CK(cudaMemcpyAsync(hcs.data(), a.cs, cs.size() * sizeof(ColState), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(ctx->hts, a.ts, nt * sizeof(TileState), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        bool capped = false;
        for (int t = 0; t < nt; t++) {
            const TileState& S = ctx->hts[t];
            ctx->stamp[t] = S.stamp + (int)std::max<long long>(0, (long long)ctx->hstats->iters - S.t0) + 4;
            if (S.done == SLOT_LIVE) capped = true;
            const TileDef& td = tiles[t0 + t];
            for (int c = 0; c < (int)td.qs.size(); c++) {
                const ColState& C = hcs[(size_t)t * W + c];
                int64_t q = td.qs[c];
                double oper;
                if (method == M_GLOBAL_GD || method == M_GLOBAL_CHEBY) oper = (double)C.rounds * ((double)n + m_vol);
                else if (method == M_HK_GLOBAL)
                    oper = (double)(relax ? C.sweep_sum : (int64_t)C.rounds) * (m_vol + (double)n);
                else if (method == M_HK_TAYLOR) oper = 0.0;
                else oper = C.oper;
                if (oper_out) oper_out[q] = oper;
                if (rounds_out) rounds_out[q] = C.rounds;
                if (lat_ms_out)
                    lat_ms_out[q] = C.finish_ns > ctx->hstats->start_ns
                                        ? (float)((double)(C.finish_ns - ctx->hstats->start_ns) * 1e-6)
                                        : 0.f;
            }
        }
        if (stats) { stats->tiles += nt; stats->tile_w = W; }
        if (capped) {
            CK(cudaEventRecord(ctx->ev[3], ctx->stream));
            return fail(ctx, GDE_EITERCAP, "max_rounds reached before the stopping rule held");
        }
    }
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    CK(cudaEventSynchronize(ctx->ev[3]));
    if (stats) {
        float tot = 0.f;
        cudaEventElapsedTime(&tot, ctx->ev[2], ctx->ev[3]);
        stats->total_ms = tot;
        stats->kernel_ms = kernel_ms;
    }
    return GDE_OK;
}

// ---------------------------------------------------------------------------
// Feature push (InstantGNN)
// ---------------------------------------------------------------------------
static int feature_push_impl(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t F, void* Pm, void* Rm,
                             int64_t ld, double eps, const int32_t* cand, int64_t ncand, bool cand_on_device,
                             double* oper_out, gde_stats* stats) {
    const int64_t n = G->g.n;
    const int prec64 = (p->prec == GDE_FP64);
    const int kind = p->kind;
    if (kind != KIND_IGN && kind != KIND_UPPR) return fail(ctx, GDE_EINVAL, "feature push needs GDE_IGN or GDE_UPPR");
    if (F <= 0 || ld < F || !Pm || !Rm) return fail(ctx, GDE_EINVAL, "bad feature matrix arguments");
    if (!(eps > 0.0)) return fail(ctx, GDE_EINVAL, "eps must be > 0");
    if (kind == KIND_IGN && (std::isnan(G->ign_beta) || G->ign_beta != p->beta)) {
        int rc = upload_ign_tables(ctx, G, p->beta);
        if (rc != GDE_OK) return rc;
    }
    if (p->omega != 0.0 && p->omega != 1.0) {
        // relaxation omega != 1: instantGNNSorPush / update_ppr's push in
        // multicolour SOR order
        if (G->relabeled) return fail(ctx, GDE_EINVAL, "the SOR feature push runs on padded (row_len) graphs");
        const int32_t* dc = cand;
        if (cand && !cand_on_device) {
            int32_t* d = (int32_t*)wsget(ctx, "sor_cand", std::max<int64_t>(ncand, 1) * 4);
            if (!d) return fail(ctx, GDE_ENOMEM, "candidate list");
            CK(cudaMemcpyAsync(d, cand, ncand * 4, cudaMemcpyHostToDevice, ctx->stream));
            dc = d;
        }
        G->g.nfac = G->nfac;
        return gde_internal_sor_feature_push(ctx, G, p, F, Pm, Rm, ld, eps, dc, ncand, oper_out, stats);
    }
    int W = p->tile_w;
    if (W <= 0) W = 8;  // 8 columns per tile (FP32: four blocks per SM); narrower and wider measured slower
    while (W > 1 && (F % W != 0 || ld % W != 0)) W >>= 1;
    if (!valid_w(W)) return fail(ctx, GDE_EINVAL, "tile_w must be 1, 2, 4, 8, 16 or 32");
    const int nt_total = (int)(F / W);
    PushArgs base{};
    fill_tuning(p, base);
    double kernel_ms = 0.0;
    if (stats) memset(stats, 0, sizeof(*stats));
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    // Kahan compensation matrix for an FP32 solution
    float* XCm = nullptr;
    if (!prec64) {
        XCm = (float*)wsget(ctx, "XCf", (size_t)n * ld * 4);
        if (!XCm) return fail(ctx, GDE_ENOMEM, "Kahan matrix");
        CK(cudaMemsetAsync(XCm, 0, (size_t)n * ld * 4, ctx->stream));
    }
    // tiles per launch bounded by workspace memory
    size_t per_tile = (size_t)n * W * (prec64 ? 8 : 4) + (size_t)n * 4 * 6 + 4096;
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    int max_tiles = (int)std::min<size_t>(512, std::max<size_t>(1, (size_t)(freeb * 0.8) / per_tile));
    for (int t0 = 0; t0 < nt_total; t0 += max_tiles) {
        const int nt = std::min(max_tiles, nt_total - t0);
        TileWs tw;
        tw.a = base;
        int rc = alloc_tiles(ctx, G, nt, W, prec64, false, false, false, false, tw);
        if (rc != GDE_OK) return rc;
        PushArgs& a = tw.a;
        // a push that starts from a candidate list (an incremental update, a
        // reference queue) visits only touched nodes: degree edits may have
        // lowered untouched thresholds, and the reference never re-examines
        // those nodes; only the initial scan of every node may go dense
        a.allow_dense = cand ? 0 : 1;
        rc = alloc_large(ctx, G, nt, tw);
        if (rc != GDE_OK) return rc;
        const size_t es = prec64 ? 8 : 4;
        a.ld = (int)ld;
        a.tile_stride = W;
        a.R = (char*)Rm + (size_t)t0 * W * es;
        a.X = (char*)Pm + (size_t)t0 * W * es;
        a.R2 = nullptr;
        a.DX = nullptr;
        if (XCm) { a.XC = XCm + (size_t)t0 * W; a.kahan = 1; }
        std::vector<TileParams> tp(nt);
        std::vector<TileState> ts(nt);
        std::vector<ColState> cs((size_t)nt * W);
        for (int t = 0; t < nt; t++) {
            TileParams& P = tp[t];
            memset(&P, 0, sizeof(P));
            P.kind = kind;
            P.method = M_LOCAL_GD;
            P.ncols = W;
            P.alpha = p->alpha;
            P.beta = p->beta;
            P.x_gain = (kind == KIND_IGN) ? p->alpha : 1.0;
            TileState& S = ts[t];
            memset(&S, 0, sizeof(S));
            S.stamp = ctx->stamp[t];
            S.dense_next[0] = cand ? 0 : 1;
            S.cand_cnt[0] = cand ? (int)ncand : 0;
            for (int c = 0; c < W; c++) {
                ColState& C = cs[(size_t)t * W + c];
                memset(&C, 0, sizeof(C));
                C.live = 1;
                C.seed = -1;
                C.theta = (kind == KIND_IGN) ? eps : p->alpha * eps;  // pow(d,1-b)*eps ; alpha*eps*degree
            }
        }
        if (cand) {
            for (int t = 0; t < nt; t++) {
                int32_t* dst = a.cand + ((int64_t)t * 2 + 0) * n;
                CK(cudaMemcpyAsync(dst, cand, ncand * 4, cand_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                   ctx->stream));
            }
        }
        CK(cudaMemcpyAsync(a.tp, tp.data(), nt * sizeof(TileParams), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(a.ts, ts.data(), nt * sizeof(TileState), cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(a.cs, cs.data(), cs.size() * sizeof(ColState), cudaMemcpyHostToDevice, ctx->stream));
        rc = run_engine(ctx, a, prec64, W, stats, &kernel_ms);
        if (rc != GDE_OK) return rc;
        std::vector<ColState> hcs(cs.size());
        CK(cudaMemcpyAsync(hcs.data(), a.cs, cs.size() * sizeof(ColState), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(ctx->hts, a.ts, nt * sizeof(TileState), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        bool capped = false;
        for (int t = 0; t < nt; t++) {
            ctx->stamp[t] =
                ctx->hts[t].stamp + (int)std::max<long long>(0, (long long)ctx->hstats->iters - ctx->hts[t].t0) + 4;
            if (ctx->hts[t].done == SLOT_LIVE) capped = true;
            for (int c = 0; c < W; c++)
                if (oper_out) oper_out[(int64_t)(t0 + t) * W + c] = hcs[(size_t)t * W + c].oper;
        }
        if (stats) { stats->tiles += nt; stats->tile_w = W; }
        if (capped) return fail(ctx, GDE_EITERCAP, "max_rounds reached before the stopping rule held");
    }
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    CK(cudaEventSynchronize(ctx->ev[3]));
    if (stats) {
        float tot = 0.f;
        cudaEventElapsedTime(&tot, ctx->ev[2], ctx->ev[3]);
        stats->total_ms = tot;
        stats->kernel_ms = kernel_ms;
    }
    return GDE_OK;
}

int gde_feature_push(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t F, void* Pm, void* Rm, int64_t ld,
                     double eps, const int32_t* cand, int64_t ncand, double* oper_out, gde_stats* stats) {
    if (!ctx || !G || !p) return fail(ctx, GDE_EINVAL, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    if (cand)
        for (int64_t i = 0; i < ncand; i++)
            if (cand[i] < 0 || cand[i] >= G->g.n) return fail(ctx, GDE_EINVAL, "candidate out of range");
    if (!G->relabeled) return feature_push_impl(ctx, G, p, F, Pm, Rm, ld, eps, cand, ncand, false, oper_out, stats);
    // relabelled static graph: run on internal-order copies of P and R
    const int64_t n = G->g.n;
    const int es = (p->prec == GDE_FP64) ? 8 : 4;
    void* Pi = wsget(ctx, "perm_P", (size_t)n * F * es);
    void* Ri = wsget(ctx, "perm_R", (size_t)n * F * es);
    if (!Pi || !Ri) return fail(ctx, GDE_ENOMEM, "permuted feature matrices");
    CK(permute_rows(Pm, ld, Pi, F, G->perm_d, n, F, es, 1, ctx->stream));
    CK(permute_rows(Rm, ld, Ri, F, G->perm_d, n, F, es, 1, ctx->stream));
    std::vector<int32_t> ci;
    if (cand) {
        ci.resize(ncand);
        for (int64_t i = 0; i < ncand; i++) ci[i] = G->h_perm[cand[i]];
    }
    int rc = feature_push_impl(ctx, G, p, F, Pi, Ri, F, eps, cand ? ci.data() : nullptr, ncand, false, oper_out, stats);
    if (rc != GDE_OK) return rc;
    // back to caller order: dst[u] = src[perm[u]]
    CK(permute_rows(Pi, F, Pm, ld, G->perm_d, n, F, es, 0, ctx->stream));
    CK(permute_rows(Ri, F, Rm, ld, G->perm_d, n, F, es, 0, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return GDE_OK;
}

int gde_plain_ppr_local(gde_ctx* ctx, gde_graph* G, int32_t seed, double alpha, double eps, float* x_out,
                        float* r_out, double* oper_out, int32_t* rounds_out) {
    if (!ctx || !G || seed < 0 || seed >= G->g.n || !(eps > 0)) return fail(ctx, GDE_EINVAL, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    const int64_t n = G->g.n;
    if (ctx->plain_n != n) {
        if (ctx->plain_n >= 0) {
            cudaFree(ctx->plain.xt); cudaFree(ctx->plain.rt); cudaFree(ctx->plain.tmp); cudaFree(ctx->plain.sp);
            cudaFree(ctx->plain.eps_vec); cudaFree(ctx->plain.queue); cudaFree(ctx->plain.nz);
            cudaFree(ctx->plain.d_count); cudaFree(ctx->plain.d_oper); cudaFreeHost(ctx->plain.h_count);
        }
        PlainWork& w = ctx->plain;
        int64_t nb = (n + 255) / 256 + 1;
        CK(cudaMalloc(&w.xt, n * 4));
        CK(cudaMalloc(&w.rt, n * 4));
        CK(cudaMalloc(&w.tmp, n * 4));
        CK(cudaMalloc(&w.sp, n * 4));
        CK(cudaMalloc(&w.eps_vec, n * 4));
        CK(cudaMalloc(&w.queue, n * 4));
        CK(cudaMalloc(&w.nz, nb * 4));
        CK(cudaMalloc(&w.d_count, 4));
        CK(cudaMalloc(&w.d_oper, 8));
        CK(cudaMallocHost(&w.h_count, 4));
        ctx->plain_n = n;
    }
    ctx->plain.degf = G->degf;
    double oper = 0;
    int rounds = 0;
    int rc = plain_ppr_local(G->g, ctx->plain, G->node_in(seed), alpha, eps, &oper, &rounds, ctx->stream);
    if (rc != GDE_OK) return fail(ctx, rc, "plain baseline failed");
    if (G->relabeled) {
        if (x_out) CK(permute_rows(ctx->plain.xt, 1, x_out, 1, G->perm_d, n, 1, 4, 0, ctx->stream));
        if (r_out) CK(permute_rows(ctx->plain.rt, 1, r_out, 1, G->perm_d, n, 1, 4, 0, ctx->stream));
    } else {
        if (x_out) CK(cudaMemcpyAsync(x_out, ctx->plain.xt, n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
        if (r_out) CK(cudaMemcpyAsync(r_out, ctx->plain.rt, n * 4, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    if (oper_out) *oper_out = oper;
    if (rounds_out) *rounds_out = rounds;
    return GDE_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Internals shared with graph_edit.cu
// ---------------------------------------------------------------------------
int gde_internal_feature_push(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t F, void* Pm, void* Rm,
                              int64_t ld, double eps, const int32_t* d_cand, int64_t ncand, double* oper_out,
                              gde_stats* stats) {
    return feature_push_impl(ctx, G, p, F, Pm, Rm, ld, eps, d_cand, ncand, true, oper_out, stats);
}

int gde_internal_graph_refresh(gde_ctx* ctx, gde_graph* G, const int64_t* h_degree, const int64_t* pos,
                               const int32_t* val, int64_t nchg, double beta, int ign) {
    if (nchg > 0) {
        int64_t* d_pos = (int64_t*)wsget(ctx, "edit_pos", nchg * 8);
        int32_t* d_val = (int32_t*)wsget(ctx, "edit_val", nchg * 4);
        if (!d_pos || !d_val) return fail(ctx, GDE_ENOMEM, "edit buffers");
        CK(cudaMemcpyAsync(d_pos, pos, nchg * 8, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(d_val, val, nchg * 4, cudaMemcpyHostToDevice, ctx->stream));
        CK(graph_apply_entries(G->col, d_pos, d_val, nchg, ctx->stream));
    }
    for (int64_t u = 0; u < G->g.n; u++) {
        G->h_len[u] = h_degree[u];
        G->h_deg[u] = (double)h_degree[u];
    }
    int rc = upload_degrees(ctx, G);
    if (rc != GDE_OK) return rc;
    if (ign) return upload_ign_tables(ctx, G, beta);
    if (G->nfac && !std::isnan(G->ign_beta)) return upload_ign_tables(ctx, G, G->ign_beta);
    return GDE_OK;
}

// The same after an edge batch that changed the degrees of `nodes` only: the
// column entries, and the degree and InstantGNN tables of those nodes.
int gde_internal_graph_refresh_nodes(gde_ctx* ctx, gde_graph* G, const int64_t* h_degree, const int64_t* nodes,
                                     int64_t nn, const int64_t* pos, const int32_t* val, int64_t nchg, double beta,
                                     int ign) {
    // the InstantGNN tables are kept for the graph's last beta: another beta rebuilds them all;
    // tables built earlier follow every later edit, whatever the kind of the update
    if (ign && (!G->nfac || std::isnan(G->ign_beta) || G->ign_beta != beta))
        return gde_internal_graph_refresh(ctx, G, h_degree, pos, val, nchg, beta, ign);
    const bool tabs = G->nfac && !std::isnan(G->ign_beta);
    const double tb = G->ign_beta;
    if (nchg > 0) {
        int64_t* d_pos = (int64_t*)wsget(ctx, "edit_pos", nchg * 8);
        int32_t* d_val = (int32_t*)wsget(ctx, "edit_val", nchg * 4);
        if (!d_pos || !d_val) return fail(ctx, GDE_ENOMEM, "edit buffers");
        CK(cudaMemcpyAsync(d_pos, pos, nchg * 8, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(d_val, val, nchg * 4, cudaMemcpyHostToDevice, ctx->stream));
        CK(graph_apply_entries(G->col, d_pos, d_val, nchg, ctx->stream));
    }
    if (nn == 0) return GDE_OK;
    std::vector<NodeTables> rec((size_t)nn);
    for (int64_t i = 0; i < nn; i++) {
        const int64_t u = nodes[i];
        const double d = (double)h_degree[u];
        G->g.vol += d - G->h_deg[u];
        G->h_len[u] = h_degree[u];
        G->h_deg[u] = d;
        if ((double)(float)d != d) G->g.degf_exact = 0;
        NodeTables& r = rec[i];
        r.id = (int32_t)u;
        r.len = (int32_t)h_degree[u];
        r.degd = d;
        r.nf = tabs ? std::pow(d, 1 - tb) : 0.0;  // as upload_ign_tables
        r.tf = tabs ? std::pow(d, tb) : 0.0;
    }
    NodeTables* d_rec = (NodeTables*)wsget(ctx, "edit_nodes", (size_t)nn * sizeof(NodeTables));
    if (!d_rec) return fail(ctx, GDE_ENOMEM, "edit buffers");
    CK(cudaMemcpyAsync(d_rec, rec.data(), (size_t)nn * sizeof(NodeTables), cudaMemcpyHostToDevice, ctx->stream));
    CK(node_tables(nn, d_rec, G->row_len, G->degd, G->degf, tabs ? G->nfac : nullptr, tabs ? G->tfac : nullptr,
                   tabs ? G->tfac_f : nullptr, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));  // rec is released on return
    return GDE_OK;
}

// A padded graph's rows moved to a new layout (gde_graph_repad): the graph
// takes ownership of row_ptr and col; degrees and node tables are unchanged.
void gde_internal_graph_relayout(gde_graph* G, int64_t* row_ptr, int32_t* col, int64_t cap, const int64_t* h_indptr) {
    cudaFree(G->row_ptr);
    cudaFree(G->col);
    G->row_ptr = row_ptr;
    G->col = col;
    G->g.row_ptr = row_ptr;
    G->g.col = col;
    G->g.cap = cap;
    G->h_indptr.assign(h_indptr, h_indptr + G->g.n + 1);
}

int gde_internal_graph_host(gde_graph* G, const int64_t** indptr, const int64_t** len, int64_t* n) {
    *indptr = G->h_indptr.data();
    *len = G->h_len.data();
    *n = G->g.n;
    return GDE_OK;
}

void* gde_internal_wsget(gde_ctx* ctx, const char* name, size_t bytes) { return wsget(ctx, name, bytes); }
void gde_internal_set_lam_max(gde_graph* G, double lam) { G->lam_max_est = lam; }
int gde_internal_fail(gde_ctx* ctx, int code, const char* msg) { return fail(ctx, code, msg); }
cudaStream_t gde_internal_stream(gde_ctx* ctx) { return ctx->stream; }
const double* gde_internal_npush(gde_graph* G) { return G->nfac; }
const double* gde_internal_degd(gde_graph* G) { return G->degd; }
bool gde_internal_relabeled(gde_graph* G) { return G->relabeled; }

// ---------------------------------------------------------------------------
// Internals shared with noalloc.cu
// ---------------------------------------------------------------------------
int gde_internal_device(gde_ctx* ctx) { return ctx->device; }
int gde_internal_sms(gde_ctx* ctx) { return ctx->sms; }
const DevGraph* gde_internal_devgraph(gde_graph* G) { return &G->g; }
int32_t gde_internal_node_in(gde_graph* G, int64_t u) { return G->node_in(u); }
double gde_internal_host_degree(gde_graph* G, int32_t u) { return G->h_deg[u]; }
void gde_internal_fill_tuning(const gde_params* p, PushArgs* a) { fill_tuning(p, *a); }
// katz_compute_prec's rule with nothing that allocates: the degree bound,
// then a cached spectral estimate; when neither clears FP32, FP64 (the
// Lanczos estimate gde_solve would compute needs device memory).
int gde_internal_katz_prec_noalloc(gde_graph* G, const gde_params* p) {
    if (p->kind != KIND_KATZ || p->prec == GDE_FP64) return p->prec;
    if (G->dmax < 0.0) {
        double m = 0.0;
        for (double d : G->h_deg) m = std::max(m, d);
        G->dmax = m;
    }
    if (p->alpha * G->dmax < kKatzFp64Ratio) return p->prec;
    if (std::isnan(G->lam_max_est)) return GDE_FP64;
    return (p->alpha * G->lam_max_est >= kKatzFp64Ratio) ? GDE_FP64 : p->prec;
}
int gde_internal_ign_tables(gde_ctx* ctx, gde_graph* G, double beta) {
    if (G->nfac && G->ign_beta == beta) return GDE_OK;
    return upload_ign_tables(ctx, G, beta);
}
