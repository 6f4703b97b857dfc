// noalloc.cu -- single-query PPR / Katz gradient-descent solve whose working
// memory is a fixed device array compiled into the library.
//
// Why: some callers must not allocate device memory while they serve a
// request.  A host that owns every byte of GPU memory through its own pool
// (a database or JVM process binding this library over FFI), a latency-bound
// serving loop where cudaMalloc / cudaFree would synchronise the device and
// stall every stream, and a process running close to the memory limit where an
// allocation in the middle of a request may fail, all need a solve that
// allocates nothing.  gde_solve grows a per-context workspace on demand; this
// entry point instead carves its workspace out of `g_noalloc_scratch`, a
// file-scope device array of kNoAllocScratchBytes (64 MiB), and calls no
// cudaMalloc, cudaFree or other allocating routine.
//
// Limits and rules of use:
//  * One query, one column: the push engine runs one tile of width 1 (the
//    batch path of gde_solve, not its served queue), kinds GDE_PPR and
//    GDE_KATZ, methods GDE_LOCAL_GD and GDE_GLOBAL_GD, FP32 or FP64.
//  * The graph's workspace must fit the array: about 44 bytes per node in
//    FP32 (52 in FP64) plus cap / 8 bytes for the long-row chunk list; larger
//    graphs are rejected with GDE_EINVAL and a message naming both sizes.
//  * Every call on a device shares the one array.  Calls whose GPU work
//    overlaps (other streams, other contexts on the same device, other host
//    threads) race on it and corrupt each other's results: serialise them.
//  * The array's name in host code is a host-side stand-in, not a device
//    address.  Every call looks the device address up with
//    cudaGetSymbolAddress, with the context's device current, and passes it
//    to the kernels; the first call on a device also loads the module there,
//    so make that first call before any stream capture begins.  (Looking the
//    address up on every call, rather than caching it, stays correct after
//    the host application resets the device and the module reloads.)
//  * Every device that loads the library holds the 64 MiB array until the
//    process exits, whether or not this entry point is ever called.
//  * Katz keeps gde_solve's precision rule: near its convergence radius
//    (alpha * lambda_max >= 0.9) an FP32 request computes in FP64.  The
//    largest degree settles most calls; otherwise a cached spectral estimate
//    of the graph decides (gde_katz_spectral_bounds, or an earlier gde_solve
//    of such a query, computes one).  With no estimate cached the call
//    computes in FP64, since the estimate itself needs device memory.
//  * Outputs are device pointers (x_out / r_out: n entries in caller node
//    order, FP64 when out64 else FP32); the small per-call records are copied
//    with cudaMemcpyAsync from / to host stack memory, and the call returns
//    after a stream synchronisation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "gde_common.cuh"
#include "gde_engine.h"

using namespace gde;

// internals of gde_capi.cu
int gde_internal_fail(gde_ctx* ctx, int code, const char* msg);
cudaStream_t gde_internal_stream(gde_ctx* ctx);
int gde_internal_device(gde_ctx* ctx);
int gde_internal_sms(gde_ctx* ctx);
const DevGraph* gde_internal_devgraph(gde_graph* G);
int32_t gde_internal_node_in(gde_graph* G, int64_t u);
double gde_internal_host_degree(gde_graph* G, int32_t u);
void gde_internal_fill_tuning(const gde_params* p, PushArgs* a);
int gde_internal_katz_prec_noalloc(gde_graph* G, const gde_params* p);

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;  // 64 MiB
constexpr size_t kAlign = 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the array on the current device.
int scratch_address(gde_ctx* ctx, unsigned char** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        std::string m = std::string("cudaGetSymbolAddress of the fixed scratch array: ") + cudaGetErrorString(e);
        return gde_internal_fail(ctx, GDE_ECUDA, m.c_str());
    }
    *out = (unsigned char*)p;
    return GDE_OK;
}

// Bump layout over the array: offsets first, pointers once the base is known.
struct Carve {
    size_t off = 0;
    size_t take(size_t bytes) {
        size_t o = off;
        off += (bytes + kAlign - 1) / kAlign * kAlign;
        return o;
    }
};

#define NA_CK(call)                                                                        \
    do {                                                                                   \
        cudaError_t e__ = (call);                                                          \
        if (e__ != cudaSuccess) {                                                          \
            std::string m__ = std::string(#call) + ": " + cudaGetErrorString(e__);        \
            return gde_internal_fail(ctx, GDE_ECUDA, m__.c_str());                         \
        }                                                                                  \
    } while (0)

}  // namespace

extern "C" int gde_solve_noalloc(gde_ctx* ctx, gde_graph* G, const gde_params* p, int32_t seed, double eps,
                                 void* x_out, void* r_out, int out64, double* oper_out, int32_t* rounds_out) {
    if (!ctx || !G || !p) return gde_internal_fail(ctx, GDE_EINVAL, "bad solve arguments");
    const int kind = p->kind, method = p->method;
    if (kind != KIND_PPR && kind != KIND_KATZ) return gde_internal_fail(ctx, GDE_EINVAL, "kind must be PPR or KATZ");
    if (method != M_LOCAL_GD && method != M_GLOBAL_GD)
        return gde_internal_fail(ctx, GDE_EINVAL, "method must be GDE_LOCAL_GD or GDE_GLOBAL_GD");
    const DevGraph& g = *gde_internal_devgraph(G);
    const int64_t n = g.n;
    if (seed < 0 || seed >= n) return gde_internal_fail(ctx, GDE_EINVAL, "seed out of range");
    if (!(eps > 0.0)) return gde_internal_fail(ctx, GDE_EINVAL, "eps must be > 0");
    const int32_t s_in = gde_internal_node_in(G, seed);
    if (kind == KIND_PPR && !(eps * gde_internal_host_degree(G, s_in) <= 1.))
        return gde_internal_fail(ctx, GDE_EINVAL, "eps * degree[s_node] > 1 (ppr_solver.py:213)");
    const int prec64 = (gde_internal_katz_prec_noalloc(G, p) == GDE_FP64);
    const size_t es = prec64 ? 8 : 4;

    PushArgs a{};
    gde_internal_fill_tuning(p, &a);
    a.large_cap = g.cap / std::max(a.chunk, 1) + g.cap / std::max(a.med_max, 1) + 64;

    // ---- layout (W = 1, one tile) ----
    Carve c;
    const size_t oR = c.take(n * es), oX = c.take(n * es), oP = c.take(n * es);
    const size_t oXC = prec64 ? 0 : c.take(n * 4);
    const size_t oCand = c.take((size_t)2 * n * 4), oMark = c.take(n * 4);
    const size_t oItems = c.take(n * sizeof(PushItem));
    const size_t oLarge = c.take((size_t)a.large_cap * sizeof(PushItem));
    const size_t oTp = c.take(sizeof(TileParams)), oTs = c.take(sizeof(TileState)), oCs = c.take(sizeof(ColState));
    const size_t oIc = c.take(sizeof(InitCol)), oEc = c.take(sizeof(ExtractCol));
    const size_t oBar = c.take(sizeof(GridBarrier)), oErr = c.take(sizeof(int)), oSt = c.take(sizeof(LaunchStats));
    if (c.off > kNoAllocScratchBytes) {
        char m[256];
        snprintf(m, sizeof m,
                 "graph too large for the fixed scratch array: needs %zu bytes, the maximum is %zu (n = %lld, cap = %lld)",
                 c.off, kNoAllocScratchBytes, (long long)n, (long long)g.cap);
        return gde_internal_fail(ctx, GDE_EINVAL, m);
    }

    const int device = gde_internal_device(ctx);
    NA_CK(cudaSetDevice(device));
    unsigned char* base = nullptr;
    int rc = scratch_address(ctx, &base);
    if (rc != GDE_OK) return rc;
    cudaStream_t st = gde_internal_stream(ctx);

    a.g = g;
    a.ntiles = 1;
    a.ld = 1;
    a.tile_stride = n;
    a.R = base + oR;
    a.X = base + oX;
    a.P = base + oP;
    a.R2 = nullptr;
    a.DX = nullptr;
    a.XC = prec64 ? nullptr : (float*)(base + oXC);
    a.kahan = prec64 ? 0 : 1;
    a.cand = (int32_t*)(base + oCand);
    a.mark = (int32_t*)(base + oMark);
    a.bsmall = (PushItem*)(base + oItems);
    a.blarge = (PushItem*)(base + oLarge);
    a.tp = (TileParams*)(base + oTp);
    a.ts = (TileState*)(base + oTs);
    a.cs = (ColState*)(base + oCs);
    a.bar = (GridBarrier*)(base + oBar);
    a.err = (int*)(base + oErr);
    a.stats = (LaunchStats*)(base + oSt);
    a.serve = 0;
    a.round_budget = a.max_rounds + 1;
    a.spin_limit = 0;

    // ---- what must start at zero (or at the "untouched" mark -1) ----
    NA_CK(cudaMemsetAsync(a.R, 0, n * es, st));
    NA_CK(cudaMemsetAsync(a.X, 0, n * es, st));
    if (a.XC) NA_CK(cudaMemsetAsync(a.XC, 0, n * 4, st));
    NA_CK(cudaMemsetAsync(a.mark, 0xff, n * 4, st));
    NA_CK(cudaMemsetAsync(a.bar, 0, sizeof(GridBarrier), st));
    NA_CK(cudaMemsetAsync(a.err, 0, sizeof(int), st));
    NA_CK(cudaMemsetAsync(a.stats, 0, sizeof(LaunchStats), st));

    // ---- tile, column and seed records (same values as gde_solve) ----
    TileParams tp;
    memset(&tp, 0, sizeof tp);
    tp.kind = kind;
    tp.method = method;
    tp.ncols = 1;
    tp.alpha = p->alpha;
    tp.x_gain = 1.0;
    TileState ts;
    memset(&ts, 0, sizeof ts);
    ts.dense_next[0] = (method == M_GLOBAL_GD) ? 1 : 0;
    ts.stamp = 0;
    ColState cs;
    memset(&cs, 0, sizeof cs);
    cs.live = 1;
    cs.seed = s_in;
    cs.theta = (kind == KIND_PPR) ? eps * p->alpha : eps;  // eps * alpha * degree (PPR), eps * degree (Katz)
    InitCol ic{};
    ic.tile = 0;
    ic.col = 0;
    ic.seed = s_in;
    ic.r0 = (kind == KIND_PPR) ? p->alpha : 1.0;
    ExtractCol ec{};
    ec.tile = 0;
    ec.col = 0;
    ec.out_row = 0;
    ec.seed = (kind == KIND_KATZ) ? seed : -1;  // xt[s_node] -= 1. (katz_solver.py:243)
    ec.seed_add = -1.0;
    ec.scale = 1.0;
    ec.r_levels = 1;
    NA_CK(cudaMemcpyAsync(a.tp, &tp, sizeof tp, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(a.ts, &ts, sizeof ts, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(a.cs, &cs, sizeof cs, cudaMemcpyHostToDevice, st));
    InitCol* d_ic = (InitCol*)(base + oIc);
    ExtractCol* d_ec = (ExtractCol*)(base + oEc);
    NA_CK(cudaMemcpyAsync(d_ic, &ic, sizeof ic, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(d_ec, &ec, sizeof ec, cudaMemcpyHostToDevice, st));

    // ---- seed, push to completion, extract ----
    NA_CK(init_columns(a, prec64, 1, d_ic, 1, st));
    const int grid = engine_max_grid(prec64, 1, gde_internal_sms(ctx));
    if (grid <= 0) return gde_internal_fail(ctx, GDE_ECUDA, "push kernel does not fit on the device");
    NA_CK(engine_launch(a, prec64, 1, grid, st));
    if (x_out || r_out) NA_CK(extract_columns(a, prec64, 1, d_ec, 1, x_out, r_out, out64, n, n, 0, st));
    int herr = 0;
    ColState hcs;
    TileState hts;
    NA_CK(cudaMemcpyAsync(&herr, a.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaMemcpyAsync(&hcs, a.cs, sizeof hcs, cudaMemcpyDeviceToHost, st));
    NA_CK(cudaMemcpyAsync(&hts, a.ts, sizeof hts, cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (herr != 0) return gde_internal_fail(ctx, herr, "a device-side wait ran out of iterations (grid barrier)");
    const double oper = (method == M_GLOBAL_GD) ? (double)hcs.rounds * ((double)n + g.vol) : hcs.oper;
    if (oper_out) *oper_out = oper;
    if (rounds_out) *rounds_out = hcs.rounds;
    if (hts.done == SLOT_LIVE)
        return gde_internal_fail(ctx, GDE_EITERCAP, "max_rounds reached before the stopping rule held");
    return GDE_OK;
}
