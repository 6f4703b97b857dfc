// sor_engine.cu -- LocalSOR / APPR on the GPU in multicolour order.
//
// The reference's ppr_sor / katz_sor (ppr_solver.py:331-461,
// katz_solver.py:251-337) relax nodes one at a time from a FIFO queue:
// res = omega r_u, x_u += res, r_u -= res, push (1-alpha) res / d_u (Katz:
// alpha res) to the neighbours.  A synchronous (Jacobi-order) relaxation
// diverges for the omega > 1 the reference uses (its iteration matrix
// I - omega Q has spectral radius < 1 only for omega < 2 / (2 - alpha)), so the
// GPU keeps a Gauss-Seidel order instead: a proper colouring of the graph, and
// sweeps over the colours.  In colour c's phase every pending node of colour c
// with |r_u| >= eps_vec[u] relaxes at once -- equivalent to relaxing them one
// after another, since no two of them are adjacent.  A node becomes pending
// when an addition leaves |r_v| >= eps_vec[v] (the reference's enqueue test)
// or its own update leaves it there, and is relaxed at the next phase of its
// colour.  The local solve stops after a sweep that leaves nothing pending;
// the global one relaxes every node of each colour and stops after a sweep
// with no node at or above threshold.
//
// One persistent cooperative launch runs all queries (one residual vector
// each) through the sweeps; per colour it has two phases separated by the
// bounded grid barrier: RELAX (pending nodes of the colour: test, update x and
// r, write push values) and PUSH (one warp per relaxed node's row, atomic
// residual updates, pending appends).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gde_common.cuh"
#include "gde_device.cuh"
#include "gde_engine.h"
#include "gde_internal.h"

using namespace gde;

int gde_internal_fail(gde_ctx* ctx, int code, const char* msg);
void* gde_internal_wsget(gde_ctx* ctx, const char* name, size_t bytes);

namespace {

constexpr int kSorThreads = 256;

struct SorArgs {
    DevGraph g;
    int nq;
    int ncolors;
    int local;
    int katz;
    int ign;                 // feature columns: 1 InstantGNN (thresholds eps d^(1-beta), target scale d^-beta),
                             // 2 dynamic PPR (update_ppr: thresholds alpha eps d); both absorb lone nodes
    double alpha, omega;
    const int32_t* color;    // [n] internal ids
    const int32_t* corder;   // [n] nodes sorted by colour
    const int32_t* cstart;   // [C+1]
    void* R;                 // [nq][n] residual (T)
    double* X;               // [nq][n] solution
    int32_t* plist;          // [nq][2][n] pending lists, colour c at [cstart[c], cstart[c+1])
    int* pcnt;               // [nq][2][C]
    int32_t* mark;           // [nq][n] 1 while pending
    int32_t* front;          // [nq][n] nodes relaxed in this phase
    void* pv;                // [nq][n] their push values (T)
    int* fcnt;               // [nq][2] by phase parity
    unsigned long long* gcnt;// [nq][2] global: nodes at or above threshold after a sweep
    const double* theta;     // [nq]
    double* oper;            // [nq]
    int* sweeps;             // [nq]
    int* done;               // [nq]
    int max_sweeps;
    GridBarrier* bar;
    int* err;
};

template <typename T>
__device__ __forceinline__ bool at_or_above(T r, double theta, double d) {
    return fabs((double)r) >= theta * d;
}

// pending append of v (colour cv) into buffer b of query q
__device__ __forceinline__ void push_pending(const SorArgs& a, int q, int b, int v, int cv) {
    const int64_t n = a.g.n;
    const int slot = atomicAdd(&a.pcnt[((int64_t)q * 2 + b) * a.ncolors + cv], 1);
    a.plist[((int64_t)q * 2 + b) * n + a.cstart[cv] + slot] = v;
}

template <typename T>
__device__ void relax_phase(const SorArgs& a, int q, int c, int p, int it) {
    const int64_t n = a.g.n;
    T* R = reinterpret_cast<T*>(a.R) + (int64_t)q * n;
    double* X = a.X + (int64_t)q * n;
    T* pv = reinterpret_cast<T*>(a.pv) + (int64_t)q * n;
    int32_t* front = a.front + (int64_t)q * n;
    int32_t* mark = a.mark + (int64_t)q * n;
    int* fc = &a.fcnt[q * 2 + (it & 1)];
    const double theta = a.theta[q];
    const int lane = threadIdx.x & 31;
    const int64_t cb = a.cstart[c];
    int64_t count;
    const int32_t* list;
    if (a.local) {
        count = a.pcnt[((int64_t)q * 2 + p) * a.ncolors + c];
        list = a.plist + ((int64_t)q * 2 + p) * n + cb;
    } else {
        count = a.cstart[c + 1] - cb;
        list = a.corder + cb;
    }
    double my_oper = 0.0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < count; base += stride) {
        const int64_t i = base + threadIdx.x;
        bool act = false;
        int u = 0;
        T push = T(0);
        if (i < count) {
            u = list[i];
            if (a.local) mark[u] = 0;
            const T r = R[u];
            const double d = a.g.degd[u];
            const double tf = (a.ign == 1) ? a.g.nfac[u] : d;  // threshold factor: d, or d^(1-beta)
            act = a.local ? at_or_above(r, theta, tf) : (r != T(0));
            if (act && a.ign) {
                const int64_t rp = a.g.row_ptr[u];
                const int len = a.g.row_len[u];
                if (len == 0 || (len == 1 && a.g.col[rp] == u)) {
                    // absorbing node: p = r, r = 0 (InstantGNN.py:81-84, ppr_solver.py:802-805)
                    X[u] = (double)r;
                    R[u] = T(0);
                    act = false;
                }
            }
            if (act && a.ign == 1) {
                // InstantGNN.py:85-88
                const double res = a.omega * (double)r;
                X[u] += a.alpha * res;
                const T rn = (T)((1 - a.omega) * (double)r);
                R[u] = rn;
                push = (T)(((1. - a.alpha) * res) / a.g.npush[u]);
                my_oper += d;
                if (at_or_above(rn, theta, tf)) {  // :94-97
                    mark[u] = 1;
                    push_pending(a, q, p ^ 1, u, c);
                }
            } else if (act) {
                // ppr_solver.py:390-395 / katz_solver.py:296-301; update_ppr: ppr_solver.py:806-813
                const double res = a.omega * (double)r;
                X[u] += res;
                const T rn = (T)((double)r - res);
                R[u] = rn;
                push = (T)(a.katz ? a.alpha * res : ((1. - a.alpha) * res) / d);
                my_oper += d;
                if (a.local && at_or_above(rn, theta, d)) {  // put u back (:402-405)
                    mark[u] = 1;
                    push_pending(a, q, p ^ 1, u, c);
                }
            }
        }
        const unsigned b = __ballot_sync(0xffffffffu, act);
        if (b) {
            int slot = 0;
            if (lane == 0) slot = atomicAdd(fc, __popc(b));
            slot = __shfl_sync(0xffffffffu, slot, 0) + __popc(b & ((1u << lane) - 1u));
            if (act) {
                front[slot] = u;
                pv[slot] = push;
            }
        }
    }
    if (a.local && my_oper != 0.0) atomicAdd(&a.oper[q], my_oper);
}

template <typename T>
__device__ void push_phase(const SorArgs& a, int q, int c, int p, int it) {
    const int64_t n = a.g.n;
    T* R = reinterpret_cast<T*>(a.R) + (int64_t)q * n;
    const T* pv = reinterpret_cast<const T*>(a.pv) + (int64_t)q * n;
    const int32_t* front = a.front + (int64_t)q * n;
    int32_t* mark = a.mark + (int64_t)q * n;
    const int nf = a.fcnt[q * 2 + (it & 1)];
    const double theta = a.theta[q];
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t f = warp; f < nf; f += nwarps) {
        const int u = front[f];
        const T val = pv[f];
        const int64_t rp = a.g.row_ptr[u];
        const int len = a.katz ? (int)(a.g.row_ptr[u + 1] - rp) : a.g.row_len[u];
        for (int j = lane; j < len; j += 32) {
            const int v = a.g.col[rp + j];
            // InstantGNN divides by d_v^beta at the target (InstantGNN.py:90)
            const T add = (a.ign == 1) ? (T)((double)val / a.g.tfac[v]) : val;
            const T old = atomicAdd(R + v, add);
            if (a.local) {
                const T now = old + add;
                const double tf = (a.ign == 1) ? a.g.nfac[v] : a.g.degd[v];
                if (at_or_above(now, theta, tf) && mark[v] == 0 && atomicExch(&mark[v], 1) == 0) {
                    const int cv = a.color[v];
                    push_pending(a, q, (cv > c) ? p : (p ^ 1), v, cv);
                }
            }
        }
    }
}

// nodes at or above threshold after a global sweep
template <typename T>
__device__ void count_phase(const SorArgs& a, int q, int b) {
    const int64_t n = a.g.n;
    const T* R = reinterpret_cast<const T*>(a.R) + (int64_t)q * n;
    const double theta = a.theta[q];
    unsigned long long cnt = 0;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x)
        cnt += at_or_above(R[u], theta, a.g.degd[u]) ? 1ull : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&a.gcnt[q * 2 + b], cnt);
}

template <typename T>
__global__ void __launch_bounds__(kSorThreads) sor_kernel(SorArgs a) {
    __shared__ int s_live;
    __shared__ int s_work;
    const int C = a.ncolors;
    int it = 0;  // phase-pair counter (fcnt parity)
    for (int sweep = 0;; ++sweep) {
        const int p = sweep & 1;
        // ---- sweep start: which queries are still going (identical in every block) ----
        if (threadIdx.x == 0) {
            int live = 0;
            for (int q = 0; q < a.nq; ++q) {
                if (a.done[q]) continue;
                bool more;
                if (a.local) {
                    long long pend = 0;
                    for (int c = 0; c < C; ++c) pend += a.pcnt[((int64_t)q * 2 + p) * C + c];
                    more = pend > 0;
                } else {
                    more = (sweep == 0) || a.gcnt[q * 2 + (p ^ 1)] > 0;
                }
                if (!more || sweep >= a.max_sweeps) {
                    if (blockIdx.x == 0) {
                        a.done[q] = more ? 2 : 1;  // 2: stopped at max_sweeps
                        a.sweeps[q] = sweep;
                    }
                } else {
                    live = 1;
                }
            }
            s_live = live;
        }
        __syncthreads();
        if (!s_live) break;
        if (!grid_barrier(a.bar, a.err)) return;  // done flags settled before anyone moves on
        for (int c = 0; c < C; ++c) {
            // skip a colour with nothing pending in any live query (same answer in every block)
            if (threadIdx.x == 0) {
                int work = 0;
                for (int q = 0; q < a.nq && !work; ++q)
                    if (!a.done[q]) work = !a.local || a.pcnt[((int64_t)q * 2 + p) * C + c] > 0;
                s_work = work;
            }
            __syncthreads();
            if (!s_work) continue;
            for (int q = 0; q < a.nq; ++q)
                if (!a.done[q]) relax_phase<T>(a, q, c, p, it);
            if (!grid_barrier(a.bar, a.err)) return;
            for (int q = 0; q < a.nq; ++q)
                if (!a.done[q]) push_phase<T>(a, q, c, p, it);
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                for (int q = 0; q < a.nq; ++q) {
                    a.pcnt[((int64_t)q * 2 + p) * C + c] = 0;  // consumed (no PUSH appends to colour c)
                    a.fcnt[q * 2 + ((it + 1) & 1)] = 0;
                }
            }
            ++it;
            if (!grid_barrier(a.bar, a.err)) return;
        }
        if (!a.local) {
            if (blockIdx.x == 0 && threadIdx.x == 0)
                for (int q = 0; q < a.nq; ++q) a.gcnt[q * 2 + (p ^ 1)] = 0;
            if (!grid_barrier(a.bar, a.err)) return;
            for (int q = 0; q < a.nq; ++q)
                if (!a.done[q]) count_phase<T>(a, q, p);
            if (!grid_barrier(a.bar, a.err)) return;
        }
    }
}

template <typename T>
__global__ void sor_extract_kernel(const SorArgs a, int q, const int32_t* perm, int seed_caller, void* x_out,
                                   void* r_out, int out64) {
    const int64_t n = a.g.n;
    const double* X = a.X + (int64_t)q * n;
    const T* R = reinterpret_cast<const T*>(a.R) + (int64_t)q * n;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = perm ? perm[u] : u;
        double x = X[v];
        if (a.katz && u == seed_caller) x -= 1.;  // xt[s_node] -= 1. (katz_solver.py:335)
        if (x_out) {
            if (out64) reinterpret_cast<double*>(x_out)[(int64_t)q * n + u] = x;
            else reinterpret_cast<float*>(x_out)[(int64_t)q * n + u] = (float)x;
        }
        if (r_out) {
            if (out64) reinterpret_cast<double*>(r_out)[(int64_t)q * n + u] = (double)R[v];
            else reinterpret_cast<float*>(r_out)[(int64_t)q * n + u] = (float)R[v];
        }
    }
}

__global__ void sor_seed_kernel(SorArgs a, const int32_t* seeds, int prec64) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.nq) return;
    const int64_t n = a.g.n;
    const int s = seeds[q];
    const double r0 = a.katz ? 1.0 : a.alpha;
    if (prec64) reinterpret_cast<double*>(a.R)[(int64_t)q * n + s] = r0;
    else reinterpret_cast<float*>(a.R)[(int64_t)q * n + s] = (float)r0;
    if (a.local) {
        const int c = a.color[s];
        a.plist[((int64_t)q * 2 + 0) * n + a.cstart[c]] = s;
        a.pcnt[((int64_t)q * 2 + 0) * a.ncolors + c] = 1;
        a.mark[(int64_t)q * n + s] = 1;
    }
}

// Feature columns: every candidate at or above its threshold starts pending.
template <typename T>
__global__ void sor_seed_cand_kernel(SorArgs a, const int32_t* cand, int64_t ncand) {
    const int64_t n = a.g.n;
    const int64_t total = (int64_t)a.nq * ncand;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(i / ncand);
        const int64_t k = i % ncand;
        const int u = cand ? cand[k] : (int)k;
        const T r = reinterpret_cast<const T*>(a.R)[(int64_t)q * n + u];
        if (!at_or_above(r, a.theta[q], (a.ign == 1) ? a.g.nfac[u] : a.g.degd[u])) continue;
        if (atomicExch(&a.mark[(int64_t)q * n + u], 1) == 0) push_pending(a, q, 0, u, a.color[u]);
    }
}

// node-major caller matrix [n][ld] <-> per-column slabs [F][n]
template <typename T, typename S>
__global__ void sor_gather_kernel(const T* M, int64_t ld, int64_t F, int64_t n, S* slab) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * F; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = i / F, q = i % F;
        slab[q * n + u] = (S)M[u * ld + q];
    }
}
template <typename T, typename S>
__global__ void sor_scatter_kernel(const S* slab, int64_t ld, int64_t F, int64_t n, T* M) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * F; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = i / F, q = i % F;
        M[u * ld + q] = (T)slab[q * n + u];
    }
}

// Greedy proper colouring visiting nodes by descending degree (ties by
// caller id): each node takes the smallest colour no earlier neighbour has.
int build_colors(gde_graph* G) {
    const int64_t n = G->g.n;
    std::vector<int32_t> col(n, -1);
    std::vector<int64_t> seen;  // colour -> last node that saw it among its neighbours
    int C = 0;
    std::vector<int32_t> order(n);  // caller ids by descending degree (stable)
    for (int64_t u = 0; u < n; u++) order[u] = (int32_t)u;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        return G->h_len[G->node_in(a)] > G->h_len[G->node_in(b)];
    });
    // the adjacency in internal ids, from the resident graph
    std::vector<int32_t> h_col_idx(std::max<int64_t>(G->g.cap, 1));
    if (G->g.cap > 0 &&
        cudaMemcpy(h_col_idx.data(), G->col, G->g.cap * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
    for (int64_t k = 0; k < n; k++) {
        const int64_t u = G->node_in(order[k]);
        const int64_t rp = G->h_indptr[u];
        const int64_t len = G->h_len[u];
        for (int64_t j = rp; j < rp + len; j++) {
            const int32_t v = h_col_idx[j];
            if (v >= 0 && v < n && col[v] >= 0) {
                if ((int64_t)seen.size() <= col[v]) seen.resize(col[v] + 1, -1);
                seen[col[v]] = u;
            }
        }
        int c = 0;
        while (c < (int)seen.size() && seen[c] == u) c++;
        col[u] = c;
        C = std::max(C, c + 1);
    }
    G->h_color = col;
    G->ncolors = C;
    return C;
}

}  // namespace

#define SO_CK(call)                                                                       \
    do {                                                                                  \
        cudaError_t e__ = (call);                                                         \
        if (e__ != cudaSuccess) {                                                         \
            std::string m__ = std::string(#call) + ": " + cudaGetErrorString(e__);       \
            return gde_internal_fail(ctx, GDE_ECUDA, m__.c_str());                        \
        }                                                                                 \
    } while (0)

namespace {

// Workspace, colouring and per-query state of a SOR launch over nq vectors.
int sor_prepare(gde_ctx* ctx, gde_graph* G, int64_t nq, int prec64, const std::vector<double>& theta, SorArgs& a) {
    const int64_t n = G->g.n;
    cudaStream_t st = ctx->stream;
    if (G->ncolors <= 0 && build_colors(G) < 0) return gde_internal_fail(ctx, GDE_ECUDA, "reading the graph for colouring");
    const int C = G->ncolors;
    std::vector<int32_t> cstart(C + 1, 0), corder(n);
    for (int64_t u = 0; u < n; u++) cstart[G->h_color[u] + 1]++;
    for (int c = 0; c < C; c++) cstart[c + 1] += cstart[c];
    {
        std::vector<int32_t> fill(C, 0);
        for (int64_t u = 0; u < n; u++) corder[cstart[G->h_color[u]] + fill[G->h_color[u]]++] = (int32_t)u;
    }
    const size_t es = prec64 ? 8 : 4;
    auto ws = [&](const char* name, size_t bytes) { return gde_internal_wsget(ctx, name, std::max<size_t>(bytes, 8)); };
    a.g = G->g;
    a.nq = (int)nq;
    a.ncolors = C;
    int32_t* d_color = (int32_t*)ws("sor_color", n * 4);
    int32_t* d_corder = (int32_t*)ws("sor_corder", n * 4);
    int32_t* d_cstart = (int32_t*)ws("sor_cstart", (C + 1) * 4);
    a.R = ws("sor_R", (size_t)nq * n * es);
    a.X = (double*)ws("sor_X", (size_t)nq * n * 8);
    a.plist = (int32_t*)ws("sor_plist", (size_t)nq * 2 * n * 4);
    a.pcnt = (int*)ws("sor_pcnt", (size_t)nq * 2 * C * 4);
    a.mark = (int32_t*)ws("sor_mark", (size_t)nq * n * 4);
    a.front = (int32_t*)ws("sor_front", (size_t)nq * n * 4);
    a.pv = ws("sor_pv", (size_t)nq * n * es);
    a.fcnt = (int*)ws("sor_fcnt", (size_t)nq * 2 * 4);
    a.gcnt = (unsigned long long*)ws("sor_gcnt", (size_t)nq * 2 * 8);
    double* d_theta = (double*)ws("sor_theta", (size_t)nq * 8);
    a.oper = (double*)ws("sor_oper", (size_t)nq * 8);
    a.sweeps = (int*)ws("sor_sweeps", (size_t)nq * 4);
    a.done = (int*)ws("sor_done", (size_t)nq * 4);
    if (!d_color || !d_corder || !d_cstart || !a.R || !a.X || !a.plist || !a.pcnt || !a.mark || !a.front || !a.pv ||
        !a.fcnt || !a.gcnt || !d_theta || !a.oper || !a.sweeps || !a.done)
        return gde_internal_fail(ctx, GDE_ENOMEM, "device memory exhausted (SOR workspace)");
    a.color = d_color;
    a.corder = d_corder;
    a.cstart = d_cstart;
    a.theta = d_theta;
    a.bar = ctx->bar;
    a.err = ctx->derr;
    SO_CK(cudaMemcpyAsync(d_color, G->h_color.data(), n * 4, cudaMemcpyHostToDevice, st));
    SO_CK(cudaMemcpyAsync(d_corder, corder.data(), n * 4, cudaMemcpyHostToDevice, st));
    SO_CK(cudaMemcpyAsync(d_cstart, cstart.data(), (C + 1) * 4, cudaMemcpyHostToDevice, st));
    SO_CK(cudaMemcpyAsync(d_theta, theta.data(), nq * 8, cudaMemcpyHostToDevice, st));
    SO_CK(cudaMemsetAsync(a.pcnt, 0, (size_t)nq * 2 * C * 4, st));
    SO_CK(cudaMemsetAsync(a.mark, 0, (size_t)nq * n * 4, st));
    SO_CK(cudaMemsetAsync(a.fcnt, 0, (size_t)nq * 2 * 4, st));
    SO_CK(cudaMemsetAsync(a.gcnt, 0, (size_t)nq * 2 * 8, st));
    SO_CK(cudaMemsetAsync(a.oper, 0, (size_t)nq * 8, st));
    SO_CK(cudaMemsetAsync(a.done, 0, (size_t)nq * 4, st));
    SO_CK(cudaMemsetAsync(a.sweeps, 0, (size_t)nq * 4, st));
    return GDE_OK;
}

// Cooperative launch of the sweeps; per-query operation counts, sweeps and
// whether any query hit max_sweeps come back to the host.
int sor_run(gde_ctx* ctx, SorArgs& a, int prec64, std::vector<double>& hop, std::vector<int>& hsw, bool* capped,
            float* ms) {
    cudaStream_t st = ctx->stream;
    SO_CK(cudaMemsetAsync(ctx->bar, 0, sizeof(GridBarrier), st));
    SO_CK(cudaMemsetAsync(ctx->derr, 0, sizeof(int), st));
    int per_sm = 0;
    if (prec64) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sor_kernel<double>, kSorThreads, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sor_kernel<float>, kSorThreads, 0);
    const int grid = std::max(1, std::min(per_sm, 4)) * ctx->sms;
    void* args[] = {&a};
    SO_CK(cudaEventRecord(ctx->ev[0], st));
    if (prec64) SO_CK(cudaLaunchCooperativeKernel((void*)sor_kernel<double>, grid, kSorThreads, args, 0, st));
    else SO_CK(cudaLaunchCooperativeKernel((void*)sor_kernel<float>, grid, kSorThreads, args, 0, st));
    SO_CK(cudaEventRecord(ctx->ev[1], st));
    const int64_t nq = a.nq;
    hop.assign(nq, 0.0);
    hsw.assign(nq, 0);
    std::vector<int> hdone(nq);
    int herr = 0;
    SO_CK(cudaMemcpyAsync(hop.data(), a.oper, nq * 8, cudaMemcpyDeviceToHost, st));
    SO_CK(cudaMemcpyAsync(hsw.data(), a.sweeps, nq * 4, cudaMemcpyDeviceToHost, st));
    SO_CK(cudaMemcpyAsync(hdone.data(), a.done, nq * 4, cudaMemcpyDeviceToHost, st));
    SO_CK(cudaMemcpyAsync(&herr, ctx->derr, 4, cudaMemcpyDeviceToHost, st));
    SO_CK(cudaStreamSynchronize(st));
    if (herr != 0) return gde_internal_fail(ctx, herr, "a device-side wait ran out of iterations (grid barrier)");
    *capped = false;
    for (int64_t q = 0; q < nq; q++) *capped |= hdone[q] == 2;
    *ms = 0.f;
    cudaEventElapsedTime(ms, ctx->ev[0], ctx->ev[1]);
    return GDE_OK;
}

}  // namespace

extern "C" int gde_sor(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t nq, const int32_t* seeds,
                       const double* eps, int local, void* x_out, void* r_out, int out64, int out_mem, int64_t ld_out,
                       double* oper_out, int32_t* sweeps_out, gde_stats* stats) {
    if (!ctx || !G || !p || nq < 0 || (nq > 0 && (!seeds || !eps))) return gde_internal_fail(ctx, GDE_EINVAL, "bad SOR arguments");
    if (p->kind != KIND_PPR && p->kind != KIND_KATZ) return gde_internal_fail(ctx, GDE_EINVAL, "SOR kinds are PPR and Katz");
    const int64_t n = G->g.n;
    if (ld_out != n && (x_out || r_out)) return gde_internal_fail(ctx, GDE_EINVAL, "SOR outputs are dense [nq][n] (ld_out = n)");
    if (!(p->omega > 0.0 && p->omega < 2.0)) return gde_internal_fail(ctx, GDE_EINVAL, "omega must be in (0, 2)");
    for (int64_t q = 0; q < nq; q++) {
        if (seeds[q] < 0 || seeds[q] >= n) return gde_internal_fail(ctx, GDE_EINVAL, "seed out of range");
        if (!(eps[q] > 0.0)) return gde_internal_fail(ctx, GDE_EINVAL, "eps must be > 0");
        if (p->kind == KIND_PPR && !(eps[q] * G->h_deg[G->node_in(seeds[q])] <= 1.))
            return gde_internal_fail(ctx, GDE_EINVAL, "eps * degree[s_node] > 1 (ppr_solver.py:333)");
    }
    if (stats) memset(stats, 0, sizeof(*stats));
    if (nq == 0) return GDE_OK;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return gde_internal_fail(ctx, GDE_ECUDA, "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    const int prec64 = (p->prec == GDE_FP64);
    const size_t es = prec64 ? 8 : 4;
    auto ws = [&](const char* name, size_t bytes) { return gde_internal_wsget(ctx, name, std::max<size_t>(bytes, 8)); };
    std::vector<double> th(nq);
    std::vector<int32_t> sd(nq);
    for (int64_t q = 0; q < nq; q++) {
        th[q] = (p->kind == KIND_PPR) ? eps[q] * p->alpha : eps[q];
        sd[q] = G->node_in(seeds[q]);
    }
    SorArgs a{};
    int rc = sor_prepare(ctx, G, nq, prec64, th, a);
    if (rc != GDE_OK) return rc;
    a.local = local ? 1 : 0;
    a.katz = p->kind == KIND_KATZ;
    a.ign = 0;
    a.alpha = p->alpha;
    a.omega = p->omega;
    a.max_sweeps = p->max_rounds > 0 ? p->max_rounds : kDefaultMaxRounds;
    int32_t* d_seeds = (int32_t*)ws("sor_seeds", (size_t)nq * 4);
    if (!d_seeds) return gde_internal_fail(ctx, GDE_ENOMEM, "seed list");
    SO_CK(cudaMemcpyAsync(d_seeds, sd.data(), nq * 4, cudaMemcpyHostToDevice, st));
    SO_CK(cudaMemsetAsync(a.R, 0, (size_t)nq * n * es, st));
    SO_CK(cudaMemsetAsync(a.X, 0, (size_t)nq * n * 8, st));
    sor_seed_kernel<<<(int)((nq + 127) / 128), 128, 0, st>>>(a, d_seeds, prec64);
    SO_CK(cudaGetLastError());
    std::vector<double> hop;
    std::vector<int> hsw;
    bool capped = false;
    float ms = 0.f;
    rc = sor_run(ctx, a, prec64, hop, hsw, &capped, &ms);
    if (rc != GDE_OK) return rc;
    // ---- results ----
    const size_t oes = out64 ? 8 : 4;
    void* dx = nullptr;
    void* dr = nullptr;
    if (x_out) dx = (out_mem == GDE_MEM_DEVICE) ? x_out : ws("sor_xo", (size_t)nq * n * oes);
    if (r_out) dr = (out_mem == GDE_MEM_DEVICE) ? r_out : ws("sor_ro", (size_t)nq * n * oes);
    if ((x_out && !dx) || (r_out && !dr)) return gde_internal_fail(ctx, GDE_ENOMEM, "SOR output staging");
    const int eb = (int)std::min<int64_t>(1024, (n + 255) / 256);
    for (int64_t q = 0; q < nq; q++) {
        if (prec64) sor_extract_kernel<double><<<eb, 256, 0, st>>>(a, (int)q, G->g.perm, seeds[q], dx, dr, out64);
        else sor_extract_kernel<float><<<eb, 256, 0, st>>>(a, (int)q, G->g.perm, seeds[q], dx, dr, out64);
    }
    SO_CK(cudaGetLastError());
    if (out_mem != GDE_MEM_DEVICE) {
        if (x_out) SO_CK(cudaMemcpyAsync(x_out, dx, (size_t)nq * n * oes, cudaMemcpyDeviceToHost, st));
        if (r_out) SO_CK(cudaMemcpyAsync(r_out, dr, (size_t)nq * n * oes, cudaMemcpyDeviceToHost, st));
    }
    SO_CK(cudaStreamSynchronize(st));
    for (int64_t q = 0; q < nq; q++) {
        // global: every sweep touches every node and edge (ppr_solver.py:451)
        if (oper_out) oper_out[q] = local ? hop[q] : (double)hsw[q] * ((double)n + G->g.vol);
        if (sweeps_out) sweeps_out[q] = hsw[q];
    }
    if (stats) {
        stats->kernel_ms = ms;
        stats->total_ms = ms;
        stats->tiles = (int)nq;
        stats->tile_w = 1;
    }
    if (capped) return gde_internal_fail(ctx, GDE_EITERCAP, "max sweeps reached before nothing was pending");
    return GDE_OK;
}

// InstantGNN push with relaxation omega != 1 (instantGNNSorPush,
// InstantGNN.py:74-105), or update_ppr's push (ppr_solver.py:798-819) for
// GDE_UPPR, in multicolour order, on the caller's node-major device matrices
// P, R ([n][ld], F columns), in place.  Candidates: d_cand (device, ncand
// entries) or every node.
int gde_internal_sor_feature_push(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t F, void* Pm, void* Rm,
                                  int64_t ld, double eps, const int32_t* d_cand, int64_t ncand, double* oper_out,
                                  gde_stats* stats) {
    const int64_t n = G->g.n;
    if (!(p->omega > 0.0 && p->omega < 2.0)) return gde_internal_fail(ctx, GDE_EINVAL, "omega must be in (0, 2)");
    const bool uppr = (p->kind == KIND_UPPR);
    if (!uppr && !G->g.nfac) return gde_internal_fail(ctx, GDE_EINVAL, "InstantGNN tables missing");
    if (stats) memset(stats, 0, sizeof(*stats));
    if (F == 0) return GDE_OK;
    cudaStream_t st = ctx->stream;
    const int prec64 = (p->prec == GDE_FP64);
    std::vector<double> th(F, uppr ? p->alpha * eps : eps);  // alpha eps d (ppr_solver.py:832) ; eps d^(1-beta)
    SorArgs a{};
    int rc = sor_prepare(ctx, G, F, prec64, th, a);
    if (rc != GDE_OK) return rc;
    a.g = G->g;  // current tables
    a.local = 1;
    a.katz = 0;
    a.ign = uppr ? 2 : 1;
    a.alpha = p->alpha;
    a.omega = p->omega;
    a.max_sweeps = p->max_rounds > 0 ? p->max_rounds : kDefaultMaxRounds;
    const int gb = (int)std::min<int64_t>(4096, (n * F + 255) / 256);
    if (prec64) {
        sor_gather_kernel<double, double><<<gb, 256, 0, st>>>((const double*)Rm, ld, F, n, (double*)a.R);
        sor_gather_kernel<double, double><<<gb, 256, 0, st>>>((const double*)Pm, ld, F, n, a.X);
    } else {
        sor_gather_kernel<float, float><<<gb, 256, 0, st>>>((const float*)Rm, ld, F, n, (float*)a.R);
        sor_gather_kernel<float, double><<<gb, 256, 0, st>>>((const float*)Pm, ld, F, n, a.X);
    }
    const int64_t nc = d_cand ? ncand : n;
    const int sb = (int)std::min<int64_t>(4096, (nc * F + 255) / 256 + 1);
    if (prec64) sor_seed_cand_kernel<double><<<sb, 256, 0, st>>>(a, d_cand, nc);
    else sor_seed_cand_kernel<float><<<sb, 256, 0, st>>>(a, d_cand, nc);
    SO_CK(cudaGetLastError());
    std::vector<double> hop;
    std::vector<int> hsw;
    bool capped = false;
    float ms = 0.f;
    rc = sor_run(ctx, a, prec64, hop, hsw, &capped, &ms);
    if (rc != GDE_OK) return rc;
    if (prec64) {
        sor_scatter_kernel<double, double><<<gb, 256, 0, st>>>((const double*)a.R, ld, F, n, (double*)Rm);
        sor_scatter_kernel<double, double><<<gb, 256, 0, st>>>(a.X, ld, F, n, (double*)Pm);
    } else {
        sor_scatter_kernel<float, float><<<gb, 256, 0, st>>>((const float*)a.R, ld, F, n, (float*)Rm);
        sor_scatter_kernel<float, double><<<gb, 256, 0, st>>>(a.X, ld, F, n, (float*)Pm);
    }
    SO_CK(cudaGetLastError());
    SO_CK(cudaStreamSynchronize(st));
    if (oper_out)
        for (int64_t q = 0; q < F; q++) oper_out[q] = hop[q];
    if (stats) {
        stats->kernel_ms = ms;
        stats->total_ms = ms;
        stats->tiles = (int)F;
        stats->tile_w = 1;
    }
    if (capped) return gde_internal_fail(ctx, GDE_EITERCAP, "max sweeps reached before nothing was pending");
    return GDE_OK;
}

extern "C" int gde_graph_colors(gde_graph* G, int32_t* colors_out, int32_t* ncolors) {
    if (!G) return GDE_EINVAL;
    if (G->ncolors <= 0 && build_colors(G) < 0) return GDE_ECUDA;
    if (ncolors) *ncolors = G->ncolors;
    if (colors_out)
        for (int64_t u = 0; u < G->g.n; u++) colors_out[u] = G->h_color[G->node_in(u)];
    return GDE_OK;
}
