// server.cu -- online serving: queries submitted while the push kernel runs.
//
// gde_serve / gde_serve_mixed take a whole query list (with arrival times)
// before the launch.  The server here takes queries as they come: a host
// thread keeps one persistent cooperative launch of the push engine running
// while there is work, and the kernel admits every submitted query into a
// free slot at a round boundary, advances all live slots together and hands
// each finished query's row to the caller, without returning to the host.
//
//   submit  the host writes the request into a ring in pinned, mapped host
//           memory and publishes it with a release store of `tail`;
//   route   the slots run in groups with their own barriers; group 0's first
//           block reads `tail` (acquire, system scope) each of its rounds and
//           copies requests into the mailboxes of idle slots of any group;
//   admit   each group moves a mailbox request into its idle slot at its own
//           round boundary;
//   finish  the slot's solution row is gathered into the caller's row (device
//           memory or pinned host memory) by the blocks of the slot's
//           group; next round the
//           slot's vectors are cleared and the completion record is published
//           (release store of done_ticket), which gde_server_poll reads;
//   idle    after idle_ms with nothing live, draining or admitted the kernel
//           returns; the host thread launches it again on the next submit;
//   stop    the host sets the stop flag, which the kernel reads every round.
//
// The request loop of the reference is a Python loop over seeds calling the
// single-query solvers (ppr_solver.py:149-164 for ppr_gd_local_gpu); here a
// request stream feeds one resident launch.  Every device wait of the kernel
// stays bounded (grid barrier polls), and the kernel leaves on its own after
// idle_ms, so a host that stops answering never leaves it spinning.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gde_common.cuh"
#include "gde_engine.h"
#include "gde_internal.h"

using namespace gde;

int gde_internal_fail(gde_ctx* ctx, int code, const char* msg);
void gde_internal_fill_tuning(const gde_params* p, PushArgs* a);

#define CK_RET(call)                                                                                  \
    do {                                                                                              \
        cudaError_t e__ = (call);                                                                     \
        if (e__ != cudaSuccess) return fail(GDE_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
    } while (0)

namespace {

constexpr int kMaxHkLevels = 256;  // longest heat-kernel Taylor length a server accepts

// psi table of hk_sor_queue (hk_solver.py:226-229)
void psi_into(double tau, int64_t N, std::vector<double>& out) {
    std::vector<double> psi(N + 2, 1.0);
    psi[N] = 1.;
    for (int64_t i = N - 1; i >= 0; i--) psi[i] = psi[i + 1] * tau / ((double)i + 1.) + 1.;
    out.insert(out.end(), psi.begin(), psi.end());
}

// hk_solver.py:15-48 (estimate_n) in the same FP64 order
int64_t estimate_n_hk(double t, double eps) {
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

}  // namespace

struct gde_server {
    gde_ctx* ctx = nullptr;
    gde_graph* G = nullptr;
    int device = 0;
    cudaStream_t stream = nullptr;
    int S = 0;
    int prec64 = 0;
    int cap = 0;
    double tau = 0.0;
    bool hk = false;
    int grid = 0;
    PushArgs a{};
    std::vector<void*> dbufs;
    std::vector<void*> hbufs;
    // pinned, mapped host memory (host pointers; the device ones are in `a`)
    OnlineReq* h_req = nullptr;
    OnlineDone* h_done = nullptr;
    long long* h_tail = nullptr;
    long long* h_head = nullptr;
    int* h_stop = nullptr;
    TileState* h_ts = nullptr;
    std::vector<int32_t> psi_off;  // by Taylor length N (-1: none)
    double katz_alpha_fp64 = INFINITY;  // FP32 servers: Katz alpha at or above this needs FP64
    // the launching thread
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    bool stopping = false;
    std::mutex submit_mu;
    long long next_ticket = 0;
    std::atomic<int> status{GDE_OK};
    std::atomic<long long> launches{0};
    std::atomic<double> kernel_ms{0.0};
    std::string err;

    bool pending() const {
        return __atomic_load_n(h_tail, __ATOMIC_ACQUIRE) > __atomic_load_n(h_head, __ATOMIC_ACQUIRE);
    }
    void* dalloc(size_t bytes) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(bytes, 256)) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        dbufs.push_back(p);
        return p;
    }
    void* halloc(size_t bytes) {
        void* p = nullptr;
        if (cudaHostAlloc(&p, std::max<size_t>(bytes, 64), cudaHostAllocMapped) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        memset(p, 0, std::max<size_t>(bytes, 64));
        hbufs.push_back(p);
        return p;
    }
    template <typename P>
    P* dev_of(P* h) {
        void* d = nullptr;
        if (cudaHostGetDevicePointer(&d, h, 0) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return (P*)d;
    }
    void free_all() {
        for (void* p : dbufs) cudaFree(p);
        for (void* p : hbufs) cudaFreeHost(p);
        dbufs.clear();
        hbufs.clear();
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
    int fail(int code, const std::string& m) {
        err = m;
        return gde_internal_fail(ctx, code, m.c_str());
    }

    // One launch: runs until the kernel leaves (idle or stop).  Slot stamps
    // continue from the last launch (the kernel's iteration count restarts).
    int launch_once() {
        CK_RET(cudaMemsetAsync(a.bar, 0, (size_t)std::max(a.groups, 1) * sizeof(GridBarrier), stream));
        CK_RET(cudaMemsetAsync(a.err, 0, sizeof(int), stream));
        CK_RET(cudaMemsetAsync(a.stats, 0, sizeof(LaunchStats), stream));
        CK_RET(cudaMemsetAsync(a.queue.quit, 0, sizeof(int), stream));
        CK_RET(cudaMemsetAsync(a.queue.gquit, 0, (size_t)std::max(a.groups, 1) * sizeof(int), stream));
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, stream);
        launches++;  // launches started (gde_server_info)
        cudaError_t e = engine_launch(a, prec64, 1, grid, stream);
        cudaEventRecord(e1, stream);
        int herr = 0;
        LaunchStats hs{};
        if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, a.err, sizeof(int), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, a.stats, sizeof(LaunchStats), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h_ts, a.ts, S * sizeof(TileState), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        float ms = 0.f;
        if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (e != cudaSuccess) return fail(GDE_ECUDA, std::string("server launch: ") + cudaGetErrorString(e));
        launches++;
        kernel_ms = kernel_ms + (double)ms;
        // the next launch restarts its iteration count at 0: every slot's
        // stamp base moves past what this launch used, and its t0 to 0
        for (int t = 0; t < S; t++) {
            TileState& T = h_ts[t];
            T.stamp = T.stamp + (int)std::max<long long>(0, (long long)hs.iters - T.t0) + 4;
            T.t0 = 0;
        }
        CK_RET(cudaMemcpyAsync(a.ts, h_ts, S * sizeof(TileState), cudaMemcpyHostToDevice, stream));
        CK_RET(cudaStreamSynchronize(stream));
        if (herr != 0) return fail(herr, "server kernel: a device-side wait ran out of iterations (grid barrier)");
        return GDE_OK;
    }

    void run() {
        cudaSetDevice(device);
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stopping || pending(); });
                if (stopping) break;
            }
            const int rc = launch_once();
            if (rc != GDE_OK) {
                status = rc;
                break;
            }
        }
    }
};

#define CK_S(call)                                                                              \
    do {                                                                                        \
        cudaError_t e__ = (call);                                                               \
        if (e__ != cudaSuccess) {                                                               \
            int rc__ = s->fail(GDE_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
            s->free_all();                                                                      \
            delete s;                                                                           \
            return rc__;                                                                        \
        }                                                                                       \
    } while (0)

extern "C" {

int gde_server_start(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t ring_capacity, double hbm_budget_bytes,
                     double idle_ms, gde_server** out) {
    if (!ctx || !G || !p || !out) return gde_internal_fail(ctx, GDE_EINVAL, "bad server arguments");
    if (p->prec != GDE_FP32 && p->prec != GDE_FP64) return gde_internal_fail(ctx, GDE_EINVAL, "bad precision");
    if (ring_capacity < 1 || ring_capacity > (1 << 24)) return gde_internal_fail(ctx, GDE_EINVAL, "ring capacity");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return gde_internal_fail(ctx, GDE_ECUDA, "cudaSetDevice");
    gde_server* s = new gde_server();
    s->ctx = ctx;
    s->G = G;
    s->device = ctx->device;
    s->prec64 = (p->prec == GDE_FP64);
    s->cap = (int)ring_capacity;
    s->tau = p->tau;
    s->hk = p->tau >= 1.0;
    const int64_t n = G->g.n;
    PushArgs base{};
    gde_internal_fill_tuning(p, &base);
    // slots: requested (default 32, at most 512), then the HBM budget
    int S = p->slots > 0 ? p->slots : 32;
    S = std::min(S, 512);
    const int64_t es = s->prec64 ? 8 : 4;
    const int64_t large_cap = G->g.cap / std::max(base.chunk, 1) + G->g.cap / std::max(base.med_max, 1) + 64;
    const int64_t rh_bytes = s->prec64 ? 0 : std::min<int64_t>(G->g.hub_cut, (int64_t)1 << 16) * 8;
    const int64_t per_slot = n * es * (3 + (s->hk ? 1 : 0)) + (s->prec64 ? 0 : n * 4) + rh_bytes + n * 4 * 3 +
                             n * (int64_t)sizeof(PushItem) + large_cap * (int64_t)sizeof(PushItem);
    if (hbm_budget_bytes > 0.0) {
        const int64_t fit = (int64_t)(hbm_budget_bytes / (double)per_slot);
        if (fit < 1) {
            delete s;
            return gde_internal_fail(ctx, GDE_ENOMEM, "the HBM budget does not hold one query slot");
        }
        S = (int)std::min<int64_t>(S, fit);
    }
    s->S = S;
    CK_S(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    s->grid = engine_max_grid(s->prec64, 1, sms);
    if (s->grid <= 0) {
        int rc = s->fail(GDE_ECUDA, "push kernel does not fit on the device");
        s->free_all();
        delete s;
        return rc;
    }
    // ---- device workspace: S one-column slots ----
    PushArgs& a = s->a;
    a = base;
    a.g = G->g;
    a.ntiles = S;
    a.ld = 1;
    a.tile_stride = n;
    const size_t slab = (size_t)S * n * es;
    const bool inter = !s->prec64;  // FP32: interleaved {x, c} Kahan pairs
    a.R = s->dalloc(slab);
    a.X = s->dalloc(inter ? 2 * slab : slab);
    a.R2 = s->hk ? s->dalloc(slab) : nullptr;
    a.P = s->dalloc(slab);
    a.DX = nullptr;
    a.cand = (int32_t*)s->dalloc((size_t)S * 2 * n * 4);
    a.bsmall = (PushItem*)s->dalloc((size_t)S * n * sizeof(PushItem));
    a.large_cap = large_cap;
    a.blarge = (PushItem*)s->dalloc((size_t)S * large_cap * sizeof(PushItem));
    a.mark = (int32_t*)s->dalloc((size_t)S * n * 4);
    a.tp = (TileParams*)s->dalloc(S * sizeof(TileParams));
    a.ts = (TileState*)s->dalloc(S * sizeof(TileState));
    a.cs = (ColState*)s->dalloc(S * sizeof(ColState));
    a.stats = (LaunchStats*)s->dalloc(sizeof(LaunchStats));
    // Slot groups, each behind its own barrier, as in gde_serve: the default
    // is one group per slot for a PPR/Katz server and one per 8 slots for a
    // server that takes heat-kernel queries (gde_params.groups overrides).
    // Group 0 also reads the ring and places requests into idle slots of
    // every group.
    {
        const int g_default = s->hk ? std::max(1, S / 8) : S;
        a.groups = std::max(1, std::min(std::min(p->groups > 0 ? p->groups : g_default, S),
                                        std::min(kMaxGroups, s->grid)));
    }
    a.bar = (GridBarrier*)s->dalloc((size_t)a.groups * sizeof(GridBarrier));
    a.err = (int*)s->dalloc(sizeof(int));
    ServeQueue& Q = a.queue;
    Q.quit = (int*)s->dalloc(sizeof(int));
    Q.gquit = (int*)s->dalloc((size_t)a.groups * sizeof(int));
    Q.last_ns = (unsigned long long*)s->dalloc(sizeof(unsigned long long));
    Q.slot = (OnlineSlot*)s->dalloc(S * sizeof(OnlineSlot));
    bool ok = a.R && a.X && (!s->hk || a.R2) && a.P && a.cand && a.bsmall && a.blarge && a.mark && a.tp && a.ts &&
              a.cs && a.stats && a.bar && a.err && Q.quit && Q.gquit && Q.last_ns && Q.slot;
    if (!ok) {
        int rc = s->fail(GDE_ENOMEM, "device memory exhausted (server slots)");
        s->free_all();
        delete s;
        return rc;
    }
    a.xq = 0;
    a.XC = nullptr;
    a.kahan = 0;
    a.xld = 0;
    a.xtile = 0;
    if (inter) {
        a.XC = (float*)a.X + 1;
        a.xld = 2;
        a.xtile = 2 * n;
        a.kahan = 1;
    }
    a.trace = nullptr;
    a.trace_iters = 0;
    a.spin_limit = (unsigned long long)std::max<int64_t>(ctx->wait_limit, 0);
    // FP32 slots keep the residual of the highest-degree nodes in FP64
    a.RH = nullptr;
    a.rh_cut = 0;
    if (!s->prec64 && G->g.hub_cut > 0) {
        a.rh_cut = (int)std::min<int64_t>(G->g.hub_cut, (int64_t)1 << 16);
        a.RH = (double*)s->dalloc((size_t)S * a.rh_cut * 8);
        if (!a.RH) {
            int rc = s->fail(GDE_ENOMEM, "device memory exhausted (FP64 hub residuals)");
            s->free_all();
            delete s;
            return rc;
        }
    }
    a.serve = 1;
    a.round_budget = 0x7fffffff;
    // ---- heat-kernel psi tables for every Taylor length the server accepts ----
    std::vector<double> psi_all;
    s->psi_off.assign(kMaxHkLevels + 1, -1);
    if (s->hk)
        for (int N = 1; N <= kMaxHkLevels; N++) {
            s->psi_off[N] = (int32_t)psi_all.size();
            psi_into(s->tau, N, psi_all);
        }
    double* d_psi = (double*)s->dalloc(std::max<size_t>(psi_all.size(), 1) * 8);
    if (!d_psi) {
        int rc = s->fail(GDE_ENOMEM, "device memory exhausted (psi tables)");
        s->free_all();
        delete s;
        return rc;
    }
    if (!psi_all.empty())
        CK_S(cudaMemcpyAsync(d_psi, psi_all.data(), psi_all.size() * 8, cudaMemcpyHostToDevice, s->stream));
    // ---- pinned, mapped host ring ----
    s->h_req = (OnlineReq*)s->halloc((size_t)s->cap * sizeof(OnlineReq));
    s->h_done = (OnlineDone*)s->halloc((size_t)s->cap * sizeof(OnlineDone));
    s->h_tail = (long long*)s->halloc(64);
    s->h_head = (long long*)s->halloc(64);
    s->h_stop = (int*)s->halloc(64);
    s->h_ts = (TileState*)s->halloc(S * sizeof(TileState));
    if (!s->h_req || !s->h_done || !s->h_tail || !s->h_head || !s->h_stop || !s->h_ts) {
        int rc = s->fail(GDE_ENOMEM, "pinned host memory (server ring)");
        s->free_all();
        delete s;
        return rc;
    }
    for (int i = 0; i < s->cap; i++) s->h_done[i].done_ticket = -1;
    Q.online = 1;
    Q.cap = s->cap;
    Q.req = s->dev_of(s->h_req);
    Q.done = s->dev_of(s->h_done);
    Q.tail = s->dev_of(s->h_tail);
    Q.head = s->dev_of(s->h_head);
    Q.stop = s->dev_of(s->h_stop);
    if (!Q.req || !Q.done || !Q.tail || !Q.head || !Q.stop) {
        int rc = s->fail(GDE_ECUDA, "device pointers of the pinned ring");
        s->free_all();
        delete s;
        return rc;
    }
    Q.idle_ns = (unsigned long long)(std::max(idle_ms, 0.0) * 1e6);
    Q.perm = G->perm_d;
    Q.psi = d_psi;
    Q.tau = s->tau;
    Q.hk_scale = std::exp(s->tau);
    Q.nq = 0;
    // ---- every slot idle, vectors zero, marks untouched ----
    CK_S(cudaMemsetAsync(a.R, 0, slab, s->stream));
    CK_S(cudaMemsetAsync(a.X, 0, inter ? 2 * slab : slab, s->stream));
    if (a.R2) CK_S(cudaMemsetAsync(a.R2, 0, slab, s->stream));
    CK_S(cudaMemsetAsync(a.mark, 0xff, (size_t)S * n * 4, s->stream));
    if (a.RH) CK_S(cudaMemsetAsync(a.RH, 0, (size_t)S * a.rh_cut * 8, s->stream));
    CK_S(cudaMemsetAsync(Q.last_ns, 0, sizeof(unsigned long long), s->stream));
    std::vector<TileParams> tp(S);
    std::vector<ColState> cs(S);
    std::vector<OnlineSlot> os(S);
    for (int t = 0; t < S; t++) {
        memset(&tp[t], 0, sizeof(TileParams));
        tp[t].kind = KIND_PPR;
        tp[t].method = M_LOCAL_GD;
        tp[t].ncols = 1;
        tp[t].x_gain = 1.0;
        tp[t].tau = s->tau;
        TileState& T = s->h_ts[t];
        memset(&T, 0, sizeof(TileState));
        T.done = SLOT_IDLE;
        T.qid = -1;
        memset(&cs[t], 0, sizeof(ColState));
        cs[t].seed = -1;
        memset(&os[t], 0, sizeof(OnlineSlot));
        os[t].ticket = -1;
    }
    CK_S(cudaMemcpyAsync(a.tp, tp.data(), S * sizeof(TileParams), cudaMemcpyHostToDevice, s->stream));
    CK_S(cudaMemcpyAsync(a.ts, s->h_ts, S * sizeof(TileState), cudaMemcpyHostToDevice, s->stream));
    CK_S(cudaMemcpyAsync(a.cs, cs.data(), S * sizeof(ColState), cudaMemcpyHostToDevice, s->stream));
    CK_S(cudaMemcpyAsync(Q.slot, os.data(), S * sizeof(OnlineSlot), cudaMemcpyHostToDevice, s->stream));
    CK_S(cudaStreamSynchronize(s->stream));
    // FP32 servers keep one precision: Katz near its convergence radius
    // (alpha * lambda_max >= 0.9, judged as gde_solve does from the degree
    // bound or a cached spectral estimate) needs an FP64 server
    if (!s->prec64) {
        double dmax = 0.0;
        for (double d : G->h_deg) dmax = std::max(dmax, d);
        const double lam = std::isnan(G->lam_max_est) ? dmax : G->lam_max_est;
        s->katz_alpha_fp64 = lam > 0.0 ? 0.9 / lam : INFINITY;
    }
    s->th = std::thread([s] { s->run(); });
    *out = s;
    return GDE_OK;
}

int gde_server_submit(gde_server* s, int kind, int32_t seed, double eps, double alpha, void* x_out, int out64,
                      int64_t* ticket_out) {
    if (!s) return GDE_EINVAL;
    if (s->status != GDE_OK) return s->fail(s->status, "the server stopped after an error: " + s->err);
    gde_graph* G = s->G;
    const int64_t n = G->g.n;
    if (kind != KIND_PPR && kind != KIND_KATZ && kind != KIND_HK) return s->fail(GDE_EINVAL, "kind must be PPR, KATZ or HK");
    if (seed < 0 || seed >= n) return s->fail(GDE_EINVAL, "seed out of range");
    if (!(eps > 0.0)) return s->fail(GDE_EINVAL, "eps must be > 0");
    const int32_t s_in = G->node_in(seed);
    if (kind == KIND_PPR && !(eps * G->h_deg[s_in] <= 1.))
        return s->fail(GDE_EINVAL, "eps * degree[s_node] > 1 (ppr_solver.py:213)");
    if (kind == KIND_KATZ && alpha >= s->katz_alpha_fp64)
        return s->fail(GDE_EINVAL, "Katz near its convergence radius (alpha * lambda_max >= 0.9) needs an FP64 server");
    OnlineReq r{};
    r.kind = kind;
    r.seed = s_in;
    r.seed_caller = seed;
    r.out64 = out64 ? 1 : 0;
    if (kind == KIND_HK) {
        if (!s->hk) return s->fail(GDE_EINVAL, "heat-kernel queries need a server started with tau >= 1");
        const int64_t N = estimate_n_hk(s->tau, .5 * eps);  // hk_solver.py:216-218
        if (N < 1 || N > kMaxHkLevels) return s->fail(GDE_EINVAL, "heat-kernel Taylor length out of range");
        r.n_levels = (int32_t)N;
        r.psi_off = s->psi_off[N];
        r.theta = std::exp(s->tau) * eps;  // e^tau * eps * degree / N / psi (hk_solver.py:230)
        r.r0 = 1.0;
        r.alpha = 0.0;
    } else {
        r.theta = (kind == KIND_PPR) ? eps * alpha : eps;  // eps * alpha * degree (PPR), eps * degree (Katz)
        r.r0 = (kind == KIND_PPR) ? alpha : 1.0;
        r.alpha = alpha;
    }
    // the caller's row: device memory of this device, or pinned host memory the device can address
    if (x_out) {
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, x_out) != cudaSuccess) {
            cudaGetLastError();
            return s->fail(GDE_EINVAL, "x_out must be device memory or pinned host memory");
        }
        if (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged) {
            if (pa.device != s->device) return s->fail(GDE_EINVAL, "x_out is on another device");
            r.x_out = pa.devicePointer ? pa.devicePointer : x_out;
        } else if (pa.type == cudaMemoryTypeHost && pa.devicePointer) {
            r.x_out = pa.devicePointer;
        } else {
            return s->fail(GDE_EINVAL, "x_out must be device memory or pinned host memory");
        }
    }
    {
        std::lock_guard<std::mutex> lk(s->submit_mu);
        const long long t = s->next_ticket;
        if (t - __atomic_load_n(s->h_head, __ATOMIC_ACQUIRE) >= s->cap)
            return s->fail(GDE_ENOMEM, "request ring full: poll finished queries or start with a larger ring");
        r.ticket = t;
        s->h_req[t % s->cap] = r;
        __atomic_store_n(s->h_tail, t + 1, __ATOMIC_RELEASE);
        s->next_ticket = t + 1;
        if (ticket_out) *ticket_out = t;
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
    }
    s->cv.notify_one();
    return GDE_OK;
}

int gde_server_poll(gde_server* s, int64_t ticket, int* done, double* oper, int32_t* rounds, double* device_ms) {
    if (!s || !done || ticket < 0) return GDE_EINVAL;
    *done = 0;
    if (ticket >= s->next_ticket) return s->fail(GDE_ENOTFOUND, "unknown ticket");
    const OnlineDone* d = s->h_done + (ticket % s->cap);
    const long long t1 = __atomic_load_n(&d->done_ticket, __ATOMIC_ACQUIRE);
    if (t1 != ticket) {
        if (t1 > ticket) return s->fail(GDE_ENOTFOUND, "ticket's record was reused: poll within ring capacity");
        if (s->status != GDE_OK) return s->fail(s->status, "the server stopped after an error: " + s->err);
        return GDE_OK;
    }
    const double op = d->oper;
    const int32_t ro = d->rounds;
    const int32_t st = d->status;
    const unsigned long long a0 = d->admit_ns, f0 = d->finish_ns;
    std::atomic_thread_fence(std::memory_order_acquire);
    if (__atomic_load_n(&d->done_ticket, __ATOMIC_ACQUIRE) != ticket)
        return s->fail(GDE_ENOTFOUND, "ticket's record was reused: poll within ring capacity");
    *done = 1;
    if (oper) *oper = op;
    if (rounds) *rounds = ro;
    if (device_ms) *device_ms = f0 > a0 ? (double)(f0 - a0) * 1e-6 : 0.0;
    if (st != GDE_OK) return s->fail(st, "max_rounds reached before the stopping rule held");
    return GDE_OK;
}

int gde_server_poll_many(gde_server* s, const int64_t* tickets, int64_t k, int32_t* done, double* oper,
                         int32_t* rounds, double* device_ms) {
    if (!s || (k > 0 && (!tickets || !done))) return GDE_EINVAL;
    int rc = GDE_OK;
    for (int64_t i = 0; i < k; i++) {
        int d = 0;
        double o = 0.0, ms = 0.0;
        int32_t r = 0;
        const int st = gde_server_poll(s, tickets[i], &d, &o, &r, &ms);
        done[i] = d;
        if (oper) oper[i] = o;
        if (rounds) rounds[i] = r;
        if (device_ms) device_ms[i] = ms;
        if (st != GDE_OK && rc == GDE_OK) rc = st;
    }
    return rc;
}

int gde_server_info(gde_server* s, int* slots, int64_t* launches, double* kernel_ms, int64_t* submitted) {
    if (!s) return GDE_EINVAL;
    if (slots) *slots = s->S;
    if (launches) *launches = s->launches;
    if (kernel_ms) *kernel_ms = s->kernel_ms;
    if (submitted) *submitted = s->next_ticket;
    return s->status;
}

int gde_server_stop(gde_server* s, int drain, int64_t* abandoned) {
    if (!s) return GDE_EINVAL;
    if (drain) {
        // every submitted query finishes first (the kernel keeps running while they do)
        for (;;) {
            if (s->status != GDE_OK) break;
            bool all = true;
            for (long long t = std::max<long long>(0, s->next_ticket - s->cap); t < s->next_ticket && all; t++) {
                const long long dt = __atomic_load_n(&s->h_done[t % s->cap].done_ticket, __ATOMIC_ACQUIRE);
                all = dt >= t;
            }
            if (all) break;
            std::this_thread::sleep_for(std::chrono::microseconds(200));
        }
    }
    __atomic_store_n(s->h_stop, 1, __ATOMIC_RELEASE);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv.notify_one();
    if (s->th.joinable()) s->th.join();
    long long lost = 0;
    for (long long t = std::max<long long>(0, s->next_ticket - s->cap); t < s->next_ticket; t++)
        if (__atomic_load_n(&s->h_done[t % s->cap].done_ticket, __ATOMIC_ACQUIRE) < t) lost++;
    if (abandoned) *abandoned = lost;
    const int st = s->status;
    gde_ctx* ctx = s->ctx;
    std::string m = s->err;
    cudaSetDevice(s->device);
    s->free_all();
    delete s;
    if (st != GDE_OK) return gde_internal_fail(ctx, st, m.c_str());
    return GDE_OK;
}

}  // extern "C"
