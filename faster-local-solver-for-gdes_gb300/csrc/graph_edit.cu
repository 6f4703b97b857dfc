// graph_edit.cu -- dynamic padded-CSR edits and the incremental feature update.
//
// gde_feature_update = (1) apply an edge batch to the padded CSR with the
// sequential semantics of updetaGraph (InstantGNN.py:137-180, identical to
// updeta_graph at ppr_solver.py:723-766), mutating the caller's host arrays
// and the resident device graph; (2) repair P, R at the touched nodes on the
// GPU (InstantGNN.py:303-318 for InstantGNN, ppr_solver.py:776-792 for the
// beta = 0 PPR update); (3) push from the repaired nodes with the engine.
//
// Every batch runs on the device; there is no host pass.  Insert-only
// batches (device_insert) decide in parallel which edges are inserted and
// where every new entry lands, with exactly the sequential semantics.
// Batches with deletions or self-loops, and insert-only batches that find a
// row full, run as a dataflow over the edges (device_mixed_edit) in which
// each edge waits (bounded) on the previous edge of each endpoint.  An edge
// that fails (no slack for an insertion, or a self-loop insertion that would
// make a padding slot part of its row) stops the batch: the edges before it
// are applied, as the sequential pass would leave them, and its error is
// returned.  The caller's host arrays receive the same values afterwards.
#include <cuda_runtime.h>

#include <cmath>
#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "gde_common.cuh"
#include "gde_device.cuh"
#include "gde_engine.h"
#include "gde_internal.h"

using namespace gde;

// Implemented in gde_capi.cu (shared internals).
int gde_internal_feature_push(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t F, void* Pm, void* Rm,
                              int64_t ld, double eps, const int32_t* d_cand, int64_t ncand, double* oper_out,
                              gde_stats* stats);
int gde_internal_graph_refresh(gde_ctx* ctx, gde_graph* G, const int64_t* h_degree, const int64_t* pos,
                               const int32_t* val, int64_t nchg, double beta, int ign);
int gde_internal_graph_refresh_nodes(gde_ctx* ctx, gde_graph* G, const int64_t* h_degree, const int64_t* nodes,
                                     int64_t nn, const int64_t* pos, const int32_t* val, int64_t nchg, double beta,
                                     int ign);
int gde_internal_graph_host(gde_graph* G, const int64_t** indptr, const int64_t** len, int64_t* n);
void* gde_internal_wsget(gde_ctx* ctx, const char* name, size_t bytes);
int gde_internal_fail(gde_ctx* ctx, int code, const char* msg);
cudaStream_t gde_internal_stream(gde_ctx* ctx);
const double* gde_internal_npush(gde_graph* G);
const double* gde_internal_degd(gde_graph* G);
bool gde_internal_relabeled(gde_graph* G);
int gde_internal_ign_tables(gde_ctx* ctx, gde_graph* G, double beta);
void gde_internal_graph_relayout(gde_graph* G, int64_t* row_ptr, int32_t* col, int64_t cap, const int64_t* h_indptr);

namespace {

// Per-key repair factors, in the reference's operation order (from the
// device power tables of the edit, or computed by gde_feature_repair from the
// caller's keys).
struct RepairKey {
    int32_t u;
    int32_t ins_beg, ins_end;   // into nbr[]
    int32_t del_beg, del_end;   // into nbr[] (del_beg == del_end: none)
    double a1, a2, a3;          // IGN: (d/od)^(1-b), od^(1-b), d^(1-b) | UPPR: d, od, unused
    double b1, b2;              // IGN: od^b, d^b
};

template <typename T>
__global__ void repair_pass1(const RepairKey* keys, int nkeys, T* P, T* R, int64_t ld, int64_t F, int kind,
                             double alpha) {
    int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (int64_t)nkeys * F) return;
    int k = (int)(tid / F);
    int64_t c = tid % F;
    const RepairKey K = keys[k];
    int64_t o = (int64_t)K.u * ld + c;
    double p = (double)P[o], r = (double)R[o];
    if (kind == KIND_IGN) {
        // p[u] *= (d/od)^(1-b); r[u] += p[u]*(od^(1-b) - d^(1-b)) / d^(1-b) * 1 / alpha  (InstantGNN.py:304-305)
        p = p * K.a1;
        r = r + (((p * (K.a2 - K.a3)) / K.a3) * 1.) / alpha;
    } else {
        // p[u] *= d/od; r[u] += p[u]*(od - d)/d  (ppr_solver.py:777-778)
        p = p * (K.a1 / K.a2);
        r = r + (p * (K.a2 - K.a1)) / K.a1;
    }
    P[o] = (T)p;
    R[o] = (T)r;
}

template <typename T>
__global__ void repair_pass2(const RepairKey* keys, int nkeys, const int32_t* nbr, const T* P, T* R, const T* X,
                             int64_t ld, int64_t F, int kind, double alpha, const double* npush, const double* degd) {
    int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (int64_t)nkeys * F) return;
    int k = (int)(tid / F);
    int64_t c = tid % F;
    const RepairKey K = keys[k];
    int64_t o = (int64_t)K.u * ld + c;
    double r = (double)R[o];
    double dr;
    if (kind == KIND_IGN) {
        // InstantGNN.py:307-314
        dr = (((double)P[o] + alpha * r - alpha * (double)X[o]) * (K.b1 - K.b2)) / K.b2;
        for (int i = K.ins_beg; i < K.ins_end; i++) {
            int v = nbr[i];
            dr += ((1 - alpha) * (double)P[(int64_t)v * ld + c]) / (K.b2 * npush[v]);
        }
        for (int i = K.del_beg; i < K.del_end; i++) {
            int v = nbr[i];
            dr -= ((1 - alpha) * (double)P[(int64_t)v * ld + c]) / (K.b2 * npush[v]);
        }
        r += dr / alpha;
    } else {
        // ppr_solver.py:780-788
        dr = 0.;
        for (int i = K.ins_beg; i < K.ins_end; i++) {
            int v = nbr[i];
            dr += ((1 - alpha) * (double)P[(int64_t)v * ld + c]) / degd[v];
        }
        for (int i = K.del_beg; i < K.del_end; i++) {
            int v = nbr[i];
            dr -= ((1 - alpha) * (double)P[(int64_t)v * ld + c]) / degd[v];
        }
        r += dr;
    }
    R[o] = (T)r;
}

// ---------------------------------------------------------------------------
// Device-side insertion (updetaGraph with onlyinsert = True, no self-loops)
// ---------------------------------------------------------------------------
// Edge e = (u, v) of the batch is inserted iff v is not in u's row when the
// sequential pass reaches it, i.e. iff the pair {u, v} is absent from the
// graph at batch start and e is the first occurrence of {u, v} in the batch.
// A row receives its new neighbours in batch order: the j-th inserted edge
// incident to w (by batch index) lands at indptr[w] + degree[w] + j.

constexpr int kEdT = 256;
constexpr unsigned long long kEmptyKey = ~0ull;

__global__ void ins_exists_kernel(DevGraph g, const int32_t* us, const int32_t* vs, int64_t k, uint8_t* state) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t e = w0; e < k; e += nw) {
        const int u = us[e], v = vs[e];
        const int64_t rp = g.row_ptr[u];
        const int len = g.row_len[u];
        bool hit = false;
        for (int j = lane; j < len && !hit; j += 32) hit = (g.col[rp + j] == v);
        hit = __any_sync(0xffffffffu, hit);
        if (lane == 0) state[e] = hit ? 1 : 0;  // 1: present, skipped
    }
}

__device__ __forceinline__ unsigned long long pair_key(int u, int v) {
    const unsigned a = (unsigned)min(u, v), b = (unsigned)max(u, v);
    return ((unsigned long long)a << 32) | b;
}

__device__ __forceinline__ unsigned hash_slot(unsigned long long key, unsigned mask) {
    unsigned long long z = key * 0x9E3779B97F4A7C15ull;
    return (unsigned)(z >> 32) & mask;
}

// first occurrence of each absent pair: open addressing on the pair key,
// atomicMin of the batch index (probes bounded by the table size)
__global__ void ins_hash_kernel(const int32_t* us, const int32_t* vs, int64_t k, const uint8_t* state,
                                unsigned long long* keys, int* first, int* slot, unsigned mask, int* err) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < k; e += (int64_t)gridDim.x * blockDim.x) {
        if (state[e]) continue;
        const unsigned long long key = pair_key(us[e], vs[e]);
        unsigned h = hash_slot(key, mask);
        bool placed = false;
        for (unsigned probe = 0; probe <= mask; ++probe) {
            const unsigned long long old = atomicCAS(&keys[h], kEmptyKey, key);
            if (old == kEmptyKey || old == key) {
                atomicMin(&first[h], (int)e);
                slot[e] = (int)h;
                placed = true;
                break;
            }
            h = (h + 1) & mask;
        }
        if (!placed) atomicExch(err, 2);
    }
}

__global__ void ins_count_kernel(const int32_t* us, const int32_t* vs, int64_t k, uint8_t* state, const int* first,
                                 const int* slot, int* cnt) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < k; e += (int64_t)gridDim.x * blockDim.x) {
        if (state[e]) continue;
        if (first[slot[e]] != (int)e) {
            state[e] = 1;  // a repeat of an earlier inserted pair
            continue;
        }
        state[e] = 2;  // inserted
        atomicAdd(&cnt[us[e]], 1);
        atomicAdd(&cnt[vs[e]], 1);
    }
}

// exclusive scan of n ints: per-block scan, scan of block sums, add
__global__ void scan_block_kernel(const int* in, int* out, int64_t n, int* sums) {
    __shared__ int ws[kEdT / 32];
    const int64_t i = (int64_t)blockIdx.x * kEdT + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x = (i < n) ? in[i] : 0;
    int inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int w = 0; w < kEdT / 32; ++w) {
            const int t = ws[w];
            ws[w] = acc;
            acc += t;
        }
        sums[blockIdx.x] = acc;
    }
    __syncthreads();
    if (i < n) out[i] = ws[warp] + inc - x;
}

__global__ void scan_sums_kernel(int* sums, int nb, int* total) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int acc = 0;
    for (int b = 0; b < nb; ++b) {
        const int t = sums[b];
        sums[b] = acc;
        acc += t;
    }
    *total = acc;
}

__global__ void scan_add_kernel(int* out, int64_t n, const int* sums, const int* total) {
    const int64_t i = (int64_t)blockIdx.x * kEdT + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
    if (i == n) out[n] = *total;
}

__global__ void ins_capacity_kernel(DevGraph g, const int* cnt, int64_t n, int* err) {
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n; w += (int64_t)gridDim.x * blockDim.x)
        if (cnt[w] && g.row_ptr[w] + g.row_len[w] + cnt[w] > g.row_ptr[w + 1]) atomicExch(err, 1);
}

__global__ void ins_fill_kernel(const int32_t* us, const int32_t* vs, int64_t k, const uint8_t* state,
                                const int* off, int* fill, int* be, int* bo) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < k; e += (int64_t)gridDim.x * blockDim.x) {
        if (state[e] != 2) continue;
        const int u = us[e], v = vs[e];
        const int su = off[u] + atomicAdd(&fill[u], 1);
        be[su] = (int)e;
        bo[su] = v;
        const int sv = off[v] + atomicAdd(&fill[v], 1);
        be[sv] = (int)e;
        bo[sv] = u;
    }
}

// One warp per node with insertions: rank the node's new neighbours by batch
// index, write them after the old entries, update the degree tables.
__global__ void ins_write_kernel(DevGraph g, int32_t* col, int32_t* row_len, float* degf, double* degd,
                                 double* nfac, double* tfac, float* tfac_f, const double* pw1, const double* pwb,
                                 int64_t n, const int* cnt, const int* off, const int* be, const int* bo,
                                 int32_t* nbr_sorted, int64_t* pos_out) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = w0; w < n; w += nw) {
        const int c = cnt[w];
        if (c == 0) continue;
        const int base = off[w];
        const int old_len = row_len[w];
        const int64_t start = g.row_ptr[w] + old_len;
        for (int i = lane; i < c; i += 32) {
            const int ei = be[base + i];
            int rank = 0;
            for (int j = 0; j < c; ++j) rank += (be[base + j] < ei) ? 1 : 0;
            col[start + rank] = bo[base + i];
            nbr_sorted[base + rank] = bo[base + i];
            pos_out[base + rank] = start + rank;
        }
        __syncwarp();
        if (lane == 0) {
            const int d = old_len + c;
            row_len[w] = d;
            degf[w] = (float)d;
            degd[w] = (double)d;
            if (nfac && pw1) {
                nfac[w] = pw1[d];
                tfac[w] = pwb[d];
                tfac_f[w] = (float)pwb[d];
            }
        }
    }
}

__global__ void ins_flags_kernel(const int* cnt, int* flag, int64_t n) {
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n; w += (int64_t)gridDim.x * blockDim.x)
        flag[w] = cnt[w] > 0 ? 1 : 0;
}

__global__ void ins_keys_kernel(const int* cnt, const int* kidx, int64_t n, int32_t* keys) {
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n; w += (int64_t)gridDim.x * blockDim.x)
        if (cnt[w] > 0) keys[kidx[w]] = (int32_t)w;
}

// Repair factors of each touched node (InstantGNN.py:304-307 / ppr_solver.py:777-788).
// (del_cnt null: insert-only batch, no delete lists)
__global__ void ins_repair_keys_kernel(const int32_t* keys, int nkeys, const int* cnt, const int* del_cnt,
                                       const int* off, const int32_t* row_len, int kind, double beta,
                                       const double* pw1, const double* pwb, RepairKey* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nkeys; i += gridDim.x * blockDim.x) {
        const int u = keys[i];
        const int d = row_len[u];
        const int cd = del_cnt ? del_cnt[u] : 0;
        const int od = d - cnt[u] + cd;
        RepairKey K;
        K.u = u;
        K.ins_beg = off[u];
        K.ins_end = off[u] + cnt[u];
        K.del_beg = K.ins_end;
        K.del_end = K.ins_end + cd;
        if (kind == KIND_IGN) {
            K.a1 = pow((double)d / (double)od, 1.0 - beta);
            K.a2 = pw1[od];
            K.a3 = pw1[d];
            K.b1 = pwb[od];
            K.b2 = pwb[d];
        } else {
            K.a1 = (double)d;
            K.a2 = (double)od;
            K.a3 = 0.0;
            K.b1 = K.b2 = 0.0;
        }
        out[i] = K;
    }
}

int exclusive_scan(gde_ctx* ctx, const int* in, int* out, int64_t n, cudaStream_t st) {
    const int nb = (int)((n + kEdT) / kEdT);  // covers index n for the total
    int* sums = (int*)gde_internal_wsget(ctx, "ins_scan_sums", (size_t)nb * 4 + 8);
    if (!sums) return gde_internal_fail(ctx, GDE_ENOMEM, "scan scratch");
    int* total = sums + nb;
    scan_block_kernel<<<nb, kEdT, 0, st>>>(in, out, n, sums);
    scan_sums_kernel<<<1, 32, 0, st>>>(sums, nb, total);
    scan_add_kernel<<<nb, kEdT, 0, st>>>(out, n, sums, total);
    return GDE_OK;
}

// Degree-power tables d^(1-beta), d^beta for d = 0..max row capacity, with
// the host C library's pow (the same values upload_ign_tables computes).
int ensure_power_tables(gde_ctx* ctx, gde_graph* G, double beta) {
    int64_t dmax = 0;
    for (int64_t u = 0; u < G->g.n; u++) dmax = std::max(dmax, G->h_indptr[u + 1] - G->h_indptr[u]);
    if (G->pw1 && G->pw_beta == beta && G->pw_max >= dmax) return GDE_OK;
    std::vector<double> a(dmax + 1), b(dmax + 1);
    for (int64_t d = 0; d <= dmax; d++) {
        a[d] = std::pow((double)d, 1 - beta);
        b[d] = std::pow((double)d, beta);
    }
    cudaFree(G->pw1);
    cudaFree(G->pwb);
    G->pw1 = G->pwb = nullptr;
    if (cudaMalloc(&G->pw1, (dmax + 1) * 8) != cudaSuccess || cudaMalloc(&G->pwb, (dmax + 1) * 8) != cudaSuccess) {
        cudaGetLastError();
        return gde_internal_fail(ctx, GDE_ENOMEM, "degree power tables");
    }
    cudaStream_t st = gde_internal_stream(ctx);
    cudaMemcpyAsync(G->pw1, a.data(), (dmax + 1) * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(G->pwb, b.data(), (dmax + 1) * 8, cudaMemcpyHostToDevice, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return gde_internal_fail(ctx, GDE_ECUDA, "power tables upload");
    G->pw_max = dmax;
    G->pw_beta = beta;
    return GDE_OK;
}

// ---------------------------------------------------------------------------
// Batches with deletions (updetaGraph with onlyinsert = False,
// InstantGNN.py:137-180 / ppr_solver.py:723-766) on the device.  The
// reference edits sequentially: whether an edge is inserted or deleted, the
// degree-1 guards and the swap-with-last moves all depend on the earlier
// edges of the batch that share an endpoint.  Edges that share no endpoint
// commute, so the batch runs as a dataflow: an edge executes once the
// previous edge on each of its endpoints (`pu`, `pv`, found on the host) has,
// which reproduces the sequential result exactly.  A warp takes the edges
// e = w, w + W, ... in batch order and waits on their predecessors' done
// flags.  The lowest pending edge of the whole batch has all its
// predecessors done, and every block is resident (cooperative launch), so
// the batch always progresses; each flag has at most two waiters.
// ---------------------------------------------------------------------------
struct MixOp {
    int32_t u, v;    // endpoints (caller ids of the padded graph)
    int32_t pu, pv;  // the previous edge of the batch on u / on v, or -1
};

enum : uint8_t { MIX_NOOP = 0, MIX_INSERT = 1, MIX_DELETE = 2 };

constexpr int kScanVec = 8;  // 16-byte loads in flight per lane while a warp scans a row

// First position of x in col[r, r + d), or -1.  The aligned middle of the row
// is read as int4 with kScanVec loads in flight per lane (1024 entries per
// step); the unaligned head and the tail are read entry by entry.
__device__ __forceinline__ int warp_find_first(const int32_t* col, int64_t r, int d, int32_t x, int lane) {
    const int head = min(d, (int)((4 - (r & 3)) & 3));
    if (head > 0) {
        const unsigned b = __ballot_sync(0xffffffffu, lane < head && __ldcg(&col[r + lane]) == x);
        if (b) return __ffs(b) - 1;
    }
    const int4* vec = reinterpret_cast<const int4*>(col + r + head);
    const int nv = (d - head) >> 2;
    for (int i0 = 0; i0 < nv; i0 += 32 * kScanVec) {
        int4 c[kScanVec];
#pragma unroll
        for (int j = 0; j < kScanVec; ++j) {
            const int idx = i0 + 32 * j + lane;
            c[j] = idx < nv ? __ldcg(&vec[idx]) : make_int4(-1, -1, -1, -1);  // ids are >= 0
        }
#pragma unroll
        for (int j = 0; j < kScanVec; ++j) {
            const int w = c[j].x == x ? 0 : c[j].y == x ? 1 : c[j].z == x ? 2 : c[j].w == x ? 3 : 4;
            const unsigned b = __ballot_sync(0xffffffffu, w < 4);
            if (b) {
                const int src = __ffs(b) - 1;
                return head + 4 * (i0 + 32 * j + src) + __shfl_sync(0xffffffffu, w, src);
            }
        }
    }
    const int t0 = head + 4 * nv;
    if (t0 < d) {
        const unsigned b = __ballot_sync(0xffffffffu, t0 + lane < d && __ldcg(&col[r + t0 + lane]) == x);
        if (b) return t0 + __ffs(b) - 1;
    }
    return -1;
}

// Every x in col[r, r + d) becomes y (same access pattern).
__device__ __forceinline__ void warp_replace_all(int32_t* col, int64_t r, int d, int32_t x, int32_t y, int lane) {
    const int head = min(d, (int)((4 - (r & 3)) & 3));
    if (lane < head && __ldcg(&col[r + lane]) == x) col[r + lane] = y;
    const int4* vec = reinterpret_cast<const int4*>(col + r + head);
    const int nv = (d - head) >> 2;
    for (int i0 = 0; i0 < nv; i0 += 32 * kScanVec) {
        int4 c[kScanVec];
#pragma unroll
        for (int j = 0; j < kScanVec; ++j) {
            const int idx = i0 + 32 * j + lane;
            c[j] = idx < nv ? __ldcg(&vec[idx]) : make_int4(-1, -1, -1, -1);
        }
#pragma unroll
        for (int j = 0; j < kScanVec; ++j) {
            int32_t* q = col + r + head + 4 * (int64_t)(i0 + 32 * j + lane);
            if (c[j].x == x) q[0] = y;
            if (c[j].y == x) q[1] = y;
            if (c[j].z == x) q[2] = y;
            if (c[j].w == x) q[3] = y;
        }
    }
    const int t0 = head + 4 * nv;
    if (t0 + lane < d && __ldcg(&col[r + t0 + lane]) == x) col[r + t0 + lane] = y;
}

// A failing edge stops the batch: an insertion that finds no slack in its
// rows, or a self-loop insertion over a slot that holds no node id (see
// below).  The edge records (index << 8 | reason) in *fail (atomicMin, so
// the lowest failing index wins) and raises *state, which stops every
// waiter; the host then restores the touched rows and runs the prefix of
// the batch before that edge.  A wait that outlasts `poll_limit` polls sets
// GDE_EHANG in err.  Since a node's edges run in batch order, the node's
// insert and delete counters give each applied edge its rank among the
// node's insertions or deletions (rank[2e], rank[2e + 1] for u, v): the
// repair's neighbour lists come out in batch order without a sort.
//
// Self-loops (u == v) follow the sequential pass literally: a deletion moves
// u's last entry into the hole, every other u in the row takes the last
// entry too, and the degree drops by two (InstantGNN.py:159-164); an
// insertion writes u into one slot and counts two degrees (:171-174), so the
// slot after it becomes live with whatever it held.  That slot may hold a
// stale id (the sequential result is then reproduced) or the padding
// sentinel n, which the next push would read out of bounds: that edge fails
// with kFailLoopSlot instead.
constexpr unsigned long long kFailNone = ~0ull;
enum : int { kFailNoSlack = 1, kFailLoopSlot = 2 };

__global__ void mix_edit_kernel(const int64_t* row_ptr, int32_t* col, int32_t* row_len, const MixOp* ops, int k,
                                int only_insert, int64_t n, uint8_t* done, uint8_t* outcome, int* ins_cnt,
                                int* del_cnt, int* rank, int* state, unsigned long long* fail, int64_t poll_limit,
                                int* err) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int e = warp; e < k; e += nwarps) {
        const MixOp op = ops[e];
        const bool loop = op.u == op.v;
        // row starts and ends never change during the batch: load them before the wait
        const int64_t ru = row_ptr[op.u], ru_end = row_ptr[op.u + 1];
        const int64_t rv = row_ptr[op.v], rv_end = row_ptr[op.v + 1];
        int go = 1;
        if (lane == 0) {
            int64_t polls = 0;
            unsigned ns = 32;
            while ((op.pu >= 0 && !*(volatile const uint8_t*)&done[op.pu]) ||
                   (op.pv >= 0 && !*(volatile const uint8_t*)&done[op.pv])) {
                if (ld_volatile_i(err) != 0 || ld_volatile_i(state) != 0) { go = 0; break; }
                if (++polls > poll_limit) {
                    atomicCAS(err, 0, GDE_EHANG);
                    go = 0;
                    break;
                }
                __nanosleep(ns);
                ns = min(ns * 2u, 256u);
            }
        }
        if (!__shfl_sync(0xffffffffu, go, 0)) return;
        __threadfence();  // the predecessors' writes before this edge's reads
        const int du = __ldcg(&row_len[op.u]), dv = loop ? du : __ldcg(&row_len[op.v]);
        // first position of v in u's row (InstantGNN.py:153-155)
        const int found = warp_find_first(col, ru, du, op.v, lane);
        uint8_t oc = MIX_NOOP;
        int reason = 0;
        if (found >= 0) {
            if (!only_insert && du > 1 && dv > 1) {  // insert-only batches and the degree-1 guard keep it (:157-158)
                // swap-with-last in u's row; every u in v's row takes v's last entry (:159-162)
                const int32_t lastv = __ldcg(&col[rv + dv - 1]);
                if (lane == 0) col[ru + found] = __ldcg(&col[ru + du - 1]);
                warp_replace_all(col, rv, dv, op.u, lastv, lane);
                if (lane == 0) {
                    if (loop) {
                        row_len[op.u] = du - 2;  // both decrements land on u (:163-164)
                    } else {
                        row_len[op.u] = du - 1;
                        row_len[op.v] = dv - 1;
                    }
                }
                oc = MIX_DELETE;
            }
        } else if (ru + du + (loop ? 1 : 0) >= ru_end || rv + dv >= rv_end) {
            reason = kFailNoSlack;  // no slack left for the append: nothing is written
        } else if (loop && (uint64_t)(uint32_t)__ldcg(&col[ru + du + 1]) >= (uint64_t)n) {
            reason = kFailLoopSlot;
        } else {
            // append to both rows (:171-174); one slot and two degrees for a self-loop
            if (lane == 0) {
                col[ru + du] = op.v;
                col[rv + dv] = op.u;
                if (loop) {
                    row_len[op.u] = du + 2;
                } else {
                    row_len[op.u] = du + 1;
                    row_len[op.v] = dv + 1;
                }
            }
            oc = MIX_INSERT;
        }
        if (reason != 0) {
            if (lane == 0) {
                atomicMin(fail, ((unsigned long long)e << 8) | (unsigned long long)reason);
                atomicExch(state, 1);
            }
            return;
        }
        if (lane == 0 && oc != MIX_NOOP) {
            int* c = oc == MIX_INSERT ? ins_cnt : del_cnt;
            const int a = __ldcg(&c[op.u]);
            if (loop) {
                rank[2 * e] = a;
                rank[2 * e + 1] = a + 1;
                c[op.u] = a + 2;
            } else {
                const int b = __ldcg(&c[op.v]);
                rank[2 * e] = a;
                rank[2 * e + 1] = b;
                c[op.u] = a + 1;
                c[op.v] = b + 1;
            }
        }
        __threadfence();  // every lane's edit visible before the successors start
        __syncwarp();
        if (lane == 0) {
            outcome[e] = oc;
            __threadfence();
            *(volatile uint8_t*)&done[e] = 1;
        }
        __syncwarp();
    }
}

// Repair-list section of each node with insertions: its inserted neighbours,
// then its deleted ones (InstantGNN.py:298-314 walks a node's insert list and
// then its delete list).
__global__ void mix_sizes_kernel(const int* ins_cnt, const int* del_cnt, int64_t n, int* size) {
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n; w += (int64_t)gridDim.x * blockDim.x)
        size[w] = ins_cnt[w] > 0 ? ins_cnt[w] + del_cnt[w] : 0;
}

__global__ void mix_fill_kernel(const MixOp* ops, const uint8_t* outcome, const int* rank, int k, const int* ins_cnt,
                                const int* off, int32_t* nbr) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < k; e += gridDim.x * blockDim.x) {
        const uint8_t oc = outcome[e];
        if (oc == MIX_NOOP) continue;
        const MixOp op = ops[e];
        const int cu = ins_cnt[op.u], cv = ins_cnt[op.v];
        if (oc == MIX_INSERT) {
            nbr[off[op.u] + rank[2 * e]] = op.v;
            nbr[off[op.v] + rank[2 * e + 1]] = op.u;
        } else {
            if (cu > 0) nbr[off[op.u] + cu + rank[2 * e]] = op.v;
            if (cv > 0) nbr[off[op.v] + cv + rank[2 * e + 1]] = op.u;
        }
    }
}

// New degree tables of the touched nodes (row_len already edited).
__global__ void mix_tables_kernel(const int32_t* nodes, int64_t nt, const int32_t* row_len, float* degf, double* degd,
                                  double* nfac, double* tfac, float* tfac_f, const double* pw1, const double* pwb) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
        const int u = nodes[t];
        const int d = row_len[u];
        degf[u] = (float)d;
        degd[u] = (double)d;
        if (nfac && pw1) {
            nfac[u] = pw1[d];
            tfac[u] = pwb[d];
            tfac_f[u] = (float)pwb[d];
        }
    }
}

// A warp per touched node: its degree, and (buf non-null) its row's whole
// capacity packed at off[t].
__global__ void mix_gather_kernel(const int64_t* row_ptr, const int32_t* col, const int32_t* row_len,
                                  const int32_t* nodes, const int64_t* off, int64_t nt, int32_t* buf, int32_t* lens) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nw) {
        const int32_t u = nodes[t];
        if (lane == 0) lens[t] = row_len[u];
        if (!buf) continue;
        const int64_t r = row_ptr[u], c = row_ptr[u + 1] - r;
        for (int64_t i = lane; i < c; i += 32) buf[off[t] + i] = col[r + i];
    }
}

// What a device edit leaves for the repair and the push: the nodes with
// insertions (keys), their repair factors and neighbour lists, on the device.
struct DeviceEdit {
    int status = GDE_OK;
    bool fallback = false;       // device_insert only: the dataflow pass runs the batch instead
    // A failing edge (no slack for an insertion, or a self-loop insertion
    // over a slot without a node id): the edges before it are applied, its
    // error is returned after that partial edit, and nothing is pushed.
    int late_status = GDE_OK;
    const char* late_msg = nullptr;
    const int32_t* keys = nullptr;
    int nkeys = 0;
    RepairKey* rkeys = nullptr;
    const int32_t* nbr = nullptr;
    int64_t repair_nbr = 0;      // entries of the keys' neighbour lists
};

DeviceEdit device_mixed_edit(gde_ctx* ctx, gde_graph* G, int32_t* h_indices, int64_t* h_degree, const int32_t* us,
                             const int32_t* vs, int64_t k, int only_insert, int kind, double beta,
                             uint8_t* outcome) {
    DeviceEdit M;
    const int64_t n = G->g.n;
    const int64_t* indptr;
    const int64_t* hlen;
    int64_t nn;
    gde_internal_graph_host(G, &indptr, &hlen, &nn);
    cudaStream_t st = ctx->stream;
    auto ws = [&](const char* name, size_t bytes) { return gde_internal_wsget(ctx, name, std::max<size_t>(bytes, 8)); };
    MixOp* d_ops = (MixOp*)ws("mix_ops", (size_t)k * sizeof(MixOp));
    uint8_t* d_done = (uint8_t*)ws("mix_done", (size_t)k);
    uint8_t* d_out = (uint8_t*)ws("mix_out", (size_t)k);
    int* d_rank = (int*)ws("mix_rank", (size_t)k * 8);
    int* d_icnt = (int*)ws("mix_icnt", (size_t)n * 4);
    int* d_dcnt = (int*)ws("mix_dcnt", (size_t)n * 4);
    int* d_state = (int*)ws("mix_state", 16);
    unsigned long long* d_fail = (unsigned long long*)ws("mix_fail", 8);
    int32_t* d_nodes = (int32_t*)ws("mix_nodes", (size_t)std::min<int64_t>(2 * k, n) * 4);
    if (!d_ops || !d_done || !d_out || !d_rank || !d_icnt || !d_dcnt || !d_state || !d_fail || !d_nodes) {
        M.status = gde_internal_fail(ctx, GDE_ENOMEM, "edit batch buffers");
        return M;
    }
    auto ck = [&](cudaError_t e2, const char* what) {
        if (e2 != cudaSuccess && M.status == GDE_OK) M.status = gde_internal_fail(ctx, GDE_ECUDA, what);
    };
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mix_edit_kernel, kEdT, 0);
    const int64_t* row_ptr = G->g.row_ptr;
    int32_t* col = G->col;
    int32_t* rl = G->row_len;
    int* err = ctx->derr;
    // The batch runs as one dataflow pass.  If an edge fails, the rows the
    // pass touched go back to the caller's arrays (still unedited) and the
    // prefix before the lowest failing edge runs again; every edge of that
    // prefix saw exactly its sequential state, so the prefix shrinks to the
    // first edge that fails in batch order, whose error is then returned
    // after the edit of the edges before it.
    int64_t kk = k;
    std::vector<int32_t>& last = G->edit_last;  // -1 outside this function
    if ((int64_t)last.size() != n) last.assign((size_t)n, -1);
    std::vector<MixOp> ops;
    std::vector<int32_t> touched;
    for (;;) {
        // each edge's predecessor on either endpoint: the last earlier edge touching it
        ops.assign((size_t)kk, MixOp{});
        touched.clear();
        for (int64_t e = 0; e < kk; e++) {
            const int32_t u = us[e], v = vs[e];
            MixOp& op = ops[(size_t)e];
            op.u = u;
            op.v = v;
            op.pu = last[u];
            op.pv = last[v];
            if (op.pu < 0) touched.push_back(u);
            if (op.pv < 0 && v != u) touched.push_back(v);
            last[u] = last[v] = (int32_t)e;
        }
        for (const int32_t u : touched) last[u] = -1;
        const int64_t nt = (int64_t)touched.size();
        ck(cudaMemcpyAsync(d_ops, ops.data(), (size_t)kk * sizeof(MixOp), cudaMemcpyHostToDevice, st), "edit upload");
        ck(cudaMemcpyAsync(d_nodes, touched.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, st), "edit upload");
        ck(cudaMemsetAsync(d_done, 0, (size_t)kk, st), "edit init");
        ck(cudaMemsetAsync(d_icnt, 0, (size_t)n * 4, st), "edit init");
        ck(cudaMemsetAsync(d_dcnt, 0, (size_t)n * 4, st), "edit init");
        ck(cudaMemsetAsync(d_state, 0, 16, st), "edit init");
        ck(cudaMemsetAsync(d_fail, 0xff, 8, st), "edit init");
        ck(cudaMemsetAsync(ctx->derr, 0, sizeof(int), st), "edit init");
        const int64_t want = (kk * 32 + kEdT - 1) / kEdT;  // a warp per edge at most
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(per_sm, 1) * ctx->sms, want));
        int ki = (int)kk;
        int64_t nl = n;
        // a wait is bounded by the whole batch running in sequence (>= 1 us a poll)
        int64_t poll_limit = std::max<int64_t>((int64_t)1 << 22, 64 * kk);
        if (ctx->wait_limit > 0) poll_limit = ctx->wait_limit;
        void* args[] = {(void*)&row_ptr, (void*)&col,    (void*)&rl,     (void*)&d_ops,   (void*)&ki,
                        (void*)&only_insert, (void*)&nl, (void*)&d_done, (void*)&d_out,  (void*)&d_icnt,
                        (void*)&d_dcnt,  (void*)&d_rank, (void*)&d_state, (void*)&d_fail, (void*)&poll_limit,
                        (void*)&err};
        if (M.status == GDE_OK)
            ck(cudaLaunchCooperativeKernel((void*)mix_edit_kernel, dim3(grid), dim3(kEdT), args, 0, st),
               "edit launch");
        int herr = 0;
        unsigned long long hfail = kFailNone;
        ck(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st), "edit status");
        ck(cudaMemcpyAsync(&hfail, d_fail, 8, cudaMemcpyDeviceToHost, st), "edit status");
        ck(cudaStreamSynchronize(st), "edit kernel");
        if (M.status != GDE_OK) return M;
        if (herr == 0 && hfail == kFailNone) break;
        // The touched rows go back to the caller's (unedited) arrays.
        std::vector<int64_t> nodes, pos;
        std::vector<int32_t> val;
        nodes.reserve(touched.size());
        for (const int32_t u : touched) {
            nodes.push_back(u);
            for (int64_t i = indptr[u]; i < indptr[u + 1]; i++) {
                pos.push_back(i);
                val.push_back(h_indices[i]);
            }
        }
        M.status = gde_internal_graph_refresh_nodes(ctx, G, h_degree, nodes.data(), (int64_t)nodes.size(),
                                                    pos.data(), val.data(), (int64_t)pos.size(), NAN, 0);
        if (M.status != GDE_OK) return M;
        if (herr != 0) {
            M.status = gde_internal_fail(ctx, GDE_EHANG, "edit batch: a device-side wait ran out");
            return M;
        }
        kk = (int64_t)(hfail >> 8);
        if ((int)(hfail & 0xff) == kFailNoSlack) {
            M.late_status = GDE_ECAPACITY;
            M.late_msg = "padded row has no slack for an insertion";
        } else {
            M.late_status = GDE_EINVAL;
            M.late_msg = "a self-loop insertion would make a padding slot (no node id) part of the row";
        }
        if (kk == 0) return M;  // nothing before the failing edge
    }
    if (outcome) ck(cudaMemcpyAsync(outcome, d_out, (size_t)kk, cudaMemcpyDeviceToHost, st), "edit outcomes");
    const int64_t nt = (int64_t)touched.size();
    const int ki = (int)kk;
    // ---- repair lists, keys and degree tables, all on the device ----
    const int nbk = (int)std::min<int64_t>(4096, (n + kEdT - 1) / kEdT + 1);
    const int tb = (int)std::min<int64_t>(4096, (kk + kEdT - 1) / kEdT + 1);
    int* d_size = (int*)ws("mix_size", (size_t)n * 4);
    int* d_off = (int*)ws("mix_off", (size_t)(n + 1) * 4);
    int* d_flag = (int*)ws("mix_flag", (size_t)n * 4);
    int* d_kidx = (int*)ws("mix_kidx", (size_t)(n + 1) * 4);
    if (!d_size || !d_off || !d_flag || !d_kidx) {
        M.status = gde_internal_fail(ctx, GDE_ENOMEM, "edit batch buffers");
        return M;
    }
    mix_sizes_kernel<<<nbk, kEdT, 0, st>>>(d_icnt, d_dcnt, n, d_size);
    if (exclusive_scan(ctx, d_size, d_off, n, st) != GDE_OK) { M.status = GDE_ENOMEM; return M; }
    ins_flags_kernel<<<nbk, kEdT, 0, st>>>(d_icnt, d_flag, n);
    if (exclusive_scan(ctx, d_flag, d_kidx, n, st) != GDE_OK) { M.status = GDE_ENOMEM; return M; }
    int hcount[2] = {0, 0};  // list entries, keys
    ck(cudaMemcpyAsync(&hcount[0], d_off + n, 4, cudaMemcpyDeviceToHost, st), "edit counts");
    ck(cudaMemcpyAsync(&hcount[1], d_kidx + n, 4, cudaMemcpyDeviceToHost, st), "edit counts");
    ck(cudaStreamSynchronize(st), "edit counts");
    if (M.status != GDE_OK) return M;
    const int total = hcount[0], nkeys = hcount[1];
    int32_t* d_nbr = (int32_t*)ws("mix_nbr", (size_t)total * 4);
    int32_t* d_keys = (int32_t*)ws("mix_keys", (size_t)nkeys * 4);
    RepairKey* d_rk = (RepairKey*)ws("mix_rkeys", (size_t)nkeys * sizeof(RepairKey));
    if (!d_nbr || !d_keys || !d_rk) {
        M.status = gde_internal_fail(ctx, GDE_ENOMEM, "repair keys");
        return M;
    }
    mix_fill_kernel<<<tb, kEdT, 0, st>>>(d_ops, d_out, d_rank, ki, d_icnt, d_off, d_nbr);
    ins_keys_kernel<<<nbk, kEdT, 0, st>>>(d_icnt, d_kidx, n, d_keys);
    if (nkeys > 0)
        ins_repair_keys_kernel<<<(nkeys + kEdT - 1) / kEdT, kEdT, 0, st>>>(d_keys, nkeys, d_icnt, d_dcnt, d_off,
                                                                          G->row_len, kind, beta, G->pw1, G->pwb,
                                                                          d_rk);
    const bool ign = (kind == KIND_IGN);
    if (nt > 0)
        mix_tables_kernel<<<(int)std::min<int64_t>(4096, (nt + kEdT - 1) / kEdT), kEdT, 0, st>>>(
            d_nodes, nt, G->row_len, G->degf, G->degd, ign ? G->nfac : nullptr, G->tfac, G->tfac_f,
            ign ? G->pw1 : nullptr, G->pwb);
    ck(cudaGetLastError(), "edit repair lists");
    // ---- the edited rows and degrees back into the caller's host arrays ----
    // The touched rows' whole capacity (slack included, as the sequential
    // pass leaves it), gathered on the device, or the whole array when the
    // touched rows hold most of it.
    std::vector<int64_t> off((size_t)nt + 1, 0);
    for (int64_t t = 0; t < nt; t++) off[(size_t)t + 1] = off[(size_t)t] + indptr[touched[t] + 1] - indptr[touched[t]];
    const bool whole = 2 * off[(size_t)nt] > G->g.cap;
    int64_t* d_roff = (int64_t*)ws("mix_roff", (size_t)(nt + 1) * 8);
    int32_t* d_lens = (int32_t*)ws("mix_lens", (size_t)nt * 4);
    int32_t* d_buf = whole ? nullptr : (int32_t*)ws("mix_rows", (size_t)off[(size_t)nt] * 4);
    if (!d_roff || !d_lens || (!whole && !d_buf)) {
        M.status = gde_internal_fail(ctx, GDE_ENOMEM, "edit readback buffers");
        return M;
    }
    std::vector<int32_t> lens((size_t)nt);
    std::vector<int32_t> rows(whole ? 0 : (size_t)off[(size_t)nt]);
    ck(cudaMemcpyAsync(d_roff, off.data(), (size_t)(nt + 1) * 8, cudaMemcpyHostToDevice, st), "edit readback");
    const int gb = (int)std::min<int64_t>(4096, (nt * 32 + kEdT - 1) / kEdT + 1);
    mix_gather_kernel<<<gb, kEdT, 0, st>>>(row_ptr, col, rl, d_nodes, d_roff, nt, d_buf, d_lens);
    ck(cudaGetLastError(), "edit gather");
    ck(cudaMemcpyAsync(lens.data(), d_lens, (size_t)nt * 4, cudaMemcpyDeviceToHost, st), "edit readback");
    if (whole)
        ck(cudaMemcpyAsync(h_indices, col, (size_t)G->g.cap * 4, cudaMemcpyDeviceToHost, st), "edit readback");
    else
        ck(cudaMemcpyAsync(rows.data(), d_buf, (size_t)off[(size_t)nt] * 4, cudaMemcpyDeviceToHost, st),
           "edit readback");
    ck(cudaStreamSynchronize(st), "edit readback");
    if (M.status != GDE_OK) return M;
    for (int64_t t = 0; t < nt; t++) {
        const int32_t u = touched[(size_t)t];
        const int64_t d = lens[(size_t)t];
        G->g.vol += (double)(d - h_degree[u]);
        h_degree[u] = d;
        G->h_len[u] = d;
        G->h_deg[u] = (double)d;
        if (!whole)
            std::copy(rows.begin() + off[(size_t)t], rows.begin() + off[(size_t)t + 1], h_indices + indptr[u]);
    }
    M.keys = d_keys;
    M.nkeys = nkeys;
    M.rkeys = d_rk;
    M.nbr = d_nbr;
    M.repair_nbr = total;
    return M;
}

DeviceEdit device_insert(gde_ctx* ctx, gde_graph* G, int32_t* h_indices, int64_t* h_degree, const int32_t* us,
                           const int32_t* vs, int64_t k, int kind, double beta, uint8_t* outcome) {
    DeviceEdit R;
    const int64_t n = G->g.n;
    cudaStream_t st = gde_internal_stream(ctx);
    auto ws = [&](const char* name, size_t bytes) { return gde_internal_wsget(ctx, name, std::max<size_t>(bytes, 8)); };
    unsigned H = 1;
    while (H < 2 * (uint64_t)std::max<int64_t>(k, 1)) H <<= 1;
    int32_t* d_us = (int32_t*)ws("ins_us", k * 4);
    int32_t* d_vs = (int32_t*)ws("ins_vs", k * 4);
    uint8_t* d_state = (uint8_t*)ws("ins_state", k);
    int* d_slot = (int*)ws("ins_slot", k * 4);
    unsigned long long* d_hk = (unsigned long long*)ws("ins_hkeys", (size_t)H * 8);
    int* d_hf = (int*)ws("ins_hfirst", (size_t)H * 4);
    int* d_cnt = (int*)ws("ins_cnt", n * 4);
    int* d_fill = (int*)ws("ins_fill", n * 4);
    int* d_off = (int*)ws("ins_off", (n + 1) * 4);
    int* d_err = (int*)ws("ins_err", 4);
    if (!d_us || !d_vs || !d_state || !d_slot || !d_hk || !d_hf || !d_cnt || !d_fill || !d_off || !d_err) {
        R.status = gde_internal_fail(ctx, GDE_ENOMEM, "insertion scratch");
        return R;
    }
#define DI_CK(call)                                                                    \
    do {                                                                               \
        cudaError_t e__ = (call);                                                      \
        if (e__ != cudaSuccess) {                                                      \
            R.status = gde_internal_fail(ctx, GDE_ECUDA, cudaGetErrorString(e__));     \
            return R;                                                                  \
        }                                                                              \
    } while (0)
    DI_CK(cudaMemcpyAsync(d_us, us, k * 4, cudaMemcpyHostToDevice, st));
    DI_CK(cudaMemcpyAsync(d_vs, vs, k * 4, cudaMemcpyHostToDevice, st));
    DI_CK(cudaMemsetAsync(d_hk, 0xff, (size_t)H * 8, st));
    DI_CK(cudaMemsetAsync(d_hf, 0x7f, (size_t)H * 4, st));
    DI_CK(cudaMemsetAsync(d_cnt, 0, n * 4, st));
    DI_CK(cudaMemsetAsync(d_fill, 0, n * 4, st));
    DI_CK(cudaMemsetAsync(d_err, 0, 4, st));
    const int eb = (int)std::min<int64_t>(4096, (k * 32 + kEdT - 1) / kEdT + 1);
    const int tb = (int)std::min<int64_t>(4096, (k + kEdT - 1) / kEdT + 1);
    const int nbk = (int)std::min<int64_t>(4096, (n + kEdT - 1) / kEdT + 1);
    const int nwb = (int)std::min<int64_t>(4096, (n * 32 + kEdT - 1) / kEdT + 1);
    ins_exists_kernel<<<eb, kEdT, 0, st>>>(G->g, d_us, d_vs, k, d_state);
    ins_hash_kernel<<<tb, kEdT, 0, st>>>(d_us, d_vs, k, d_state, d_hk, d_hf, d_slot, H - 1, d_err);
    ins_count_kernel<<<tb, kEdT, 0, st>>>(d_us, d_vs, k, d_state, d_hf, d_slot, d_cnt);
    ins_capacity_kernel<<<nbk, kEdT, 0, st>>>(G->g, d_cnt, n, d_err);
    int herr = 0;
    DI_CK(cudaMemcpyAsync(&herr, d_err, 4, cudaMemcpyDeviceToHost, st));
    DI_CK(cudaStreamSynchronize(st));
    if (herr != 0) {
        // no slack for some insertion (or an overfull hash table): nothing was
        // written yet; the dataflow pass applies the sequential partial edit
        R.fallback = true;
        return R;
    }
    if (exclusive_scan(ctx, d_cnt, d_off, n, st) != GDE_OK) { R.status = GDE_ENOMEM; return R; }
    int total = 0;
    DI_CK(cudaMemcpyAsync(&total, d_off + n, 4, cudaMemcpyDeviceToHost, st));
    DI_CK(cudaStreamSynchronize(st));
    int* d_be = (int*)ws("ins_be", (size_t)total * 4);
    int* d_bo = (int*)ws("ins_bo", (size_t)total * 4);
    int32_t* d_nbr = (int32_t*)ws("ins_nbr", (size_t)total * 4);
    int64_t* d_pos = (int64_t*)ws("ins_pos", (size_t)total * 8);
    int* d_flag = (int*)ws("ins_flag", n * 4);
    int* d_kidx = (int*)ws("ins_kidx", (n + 1) * 4);
    if (!d_be || !d_bo || !d_nbr || !d_pos || !d_flag || !d_kidx) {
        R.status = gde_internal_fail(ctx, GDE_ENOMEM, "insertion scratch");
        return R;
    }
    ins_fill_kernel<<<tb, kEdT, 0, st>>>(d_us, d_vs, k, d_state, d_off, d_fill, d_be, d_bo);
    const bool ign = (kind == KIND_IGN);
    ins_write_kernel<<<nwb, kEdT, 0, st>>>(G->g, G->col, G->row_len, G->degf, G->degd, ign ? G->nfac : nullptr,
                                           G->tfac, G->tfac_f, ign ? G->pw1 : nullptr, G->pwb, n, d_cnt, d_off, d_be,
                                           d_bo, d_nbr, d_pos);
    ins_flags_kernel<<<nbk, kEdT, 0, st>>>(d_cnt, d_flag, n);
    if (exclusive_scan(ctx, d_flag, d_kidx, n, st) != GDE_OK) { R.status = GDE_ENOMEM; return R; }
    int nkeys = 0;
    DI_CK(cudaMemcpyAsync(&nkeys, d_kidx + n, 4, cudaMemcpyDeviceToHost, st));
    DI_CK(cudaStreamSynchronize(st));
    int32_t* d_keys = (int32_t*)ws("ins_keys", (size_t)nkeys * 4);
    RepairKey* d_rk = (RepairKey*)ws("ins_rkeys", (size_t)nkeys * sizeof(RepairKey));
    if (!d_keys || !d_rk) {
        R.status = gde_internal_fail(ctx, GDE_ENOMEM, "repair keys");
        return R;
    }
    ins_keys_kernel<<<nbk, kEdT, 0, st>>>(d_cnt, d_kidx, n, d_keys);
    if (nkeys > 0)
        ins_repair_keys_kernel<<<(nkeys + kEdT - 1) / kEdT, kEdT, 0, st>>>(d_keys, nkeys, d_cnt, nullptr, d_off,
                                                                          G->row_len, kind, beta, G->pw1, G->pwb,
                                                                          d_rk);
    DI_CK(cudaGetLastError());
    // ---- the same edit on the caller's host arrays and the host mirror ----
    std::vector<int64_t> hpos(total);
    std::vector<int32_t> hval(total);
    std::vector<int> hcnt(n);
    if (outcome) DI_CK(cudaMemcpyAsync(outcome, d_state, (size_t)k, cudaMemcpyDeviceToHost, st));
    DI_CK(cudaMemcpyAsync(hpos.data(), d_pos, (size_t)total * 8, cudaMemcpyDeviceToHost, st));
    DI_CK(cudaMemcpyAsync(hval.data(), d_nbr, (size_t)total * 4, cudaMemcpyDeviceToHost, st));
    DI_CK(cudaMemcpyAsync(hcnt.data(), d_cnt, n * 4, cudaMemcpyDeviceToHost, st));
    DI_CK(cudaStreamSynchronize(st));
#undef DI_CK
    // insert states: 2 inserted; 0 present already and 1 a repeat, both skipped
    if (outcome)
        for (int64_t e = 0; e < k; e++) outcome[e] = outcome[e] == 2 ? MIX_INSERT : MIX_NOOP;
    for (int i = 0; i < total; i++) h_indices[hpos[i]] = hval[i];
    for (int64_t w = 0; w < n; w++) {
        if (!hcnt[w]) continue;
        h_degree[w] += hcnt[w];
        G->h_len[w] = h_degree[w];
        G->h_deg[w] = (double)h_degree[w];
    }
    G->g.vol += (double)total;
    R.keys = d_keys;
    R.nkeys = nkeys;
    R.rkeys = d_rk;
    R.nbr = d_nbr;
    R.repair_nbr = total;
    return R;
}

// One warp per row: the live entries to the new place, the slack filled
// with the sentinel n.
__global__ void repad_rows_kernel(const int64_t* old_ptr, const int32_t* old_col, const int32_t* row_len,
                                  const int64_t* new_ptr, int32_t* new_col, int64_t n) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += nw) {
        const int64_t src = old_ptr[u], dst = new_ptr[u], c = new_ptr[u + 1] - dst;
        const int len = row_len[u];
        for (int64_t i = lane; i < c; i += 32) new_col[dst + i] = i < len ? old_col[src + i] : (int32_t)n;
    }
}

}  // namespace

extern "C" int gde_graph_repad(gde_ctx* ctx, gde_graph* G, int64_t min_slack, int64_t* indptr_out,
                               int32_t* indices_out, int64_t* cap_out) {
    if (!ctx || !G || !cap_out || min_slack < 0) return gde_internal_fail(ctx, GDE_EINVAL, "bad repad arguments");
    if (gde_internal_relabeled(G))
        return gde_internal_fail(ctx, GDE_EINVAL, "repad needs a padded CSR graph (upload with row_len)");
    const int64_t* indptr;
    const int64_t* hlen;
    int64_t n;
    gde_internal_graph_host(G, &indptr, &hlen, &n);
    std::vector<int64_t> ptr((size_t)n + 1, 0);
    for (int64_t u = 0; u < n; u++)
        ptr[(size_t)u + 1] = ptr[(size_t)u] + std::max(indptr[u + 1] - indptr[u], hlen[u] + min_slack);
    const int64_t cap = ptr[(size_t)n];
    *cap_out = cap;
    if (!indices_out) return GDE_OK;
    if (!indptr_out) return gde_internal_fail(ctx, GDE_EINVAL, "repad: indptr_out is NULL");
    cudaStream_t st = gde_internal_stream(ctx);
    int64_t* d_ptr = nullptr;
    int32_t* d_col = nullptr;
    if (cudaMalloc(&d_ptr, (size_t)(n + 3) * sizeof(int64_t)) != cudaSuccess ||
        cudaMalloc(&d_col, (size_t)std::max<int64_t>(cap, 1) * sizeof(int32_t)) != cudaSuccess) {
        cudaFree(d_ptr);
        cudaFree(d_col);
        cudaGetLastError();
        return gde_internal_fail(ctx, GDE_ENOMEM, "repad: device memory exhausted");
    }
    bool ok = cudaMemsetAsync(d_ptr, 0, (size_t)(n + 3) * sizeof(int64_t), st) == cudaSuccess &&
              cudaMemcpyAsync(d_ptr, ptr.data(), (size_t)(n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st) ==
                  cudaSuccess;
    if (ok && n > 0) {
        const int blocks = (int)std::min<int64_t>(8192, (n * 32 + kEdT - 1) / kEdT);
        repad_rows_kernel<<<blocks, kEdT, 0, st>>>(G->row_ptr, G->col, G->row_len, d_ptr, d_col, n);
        ok = cudaGetLastError() == cudaSuccess;
    }
    if (ok && cap > 0)
        ok = cudaMemcpyAsync(indices_out, d_col, (size_t)cap * sizeof(int32_t), cudaMemcpyDeviceToHost, st) ==
             cudaSuccess;
    if (ok) ok = cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) {
        cudaFree(d_ptr);
        cudaFree(d_col);
        return gde_internal_fail(ctx, GDE_ECUDA, "repad: copy of the rows");
    }
    std::copy(ptr.begin(), ptr.end(), indptr_out);
    gde_internal_graph_relayout(G, d_ptr, d_col, cap, ptr.data());
    return GDE_OK;
}

namespace {

}  // namespace

// The edge batch, then (unless edit_only) the repair and the push.
// outcome (host, may be null): per edge MIX_NOOP / MIX_INSERT / MIX_DELETE.
static int feature_update_impl(gde_ctx* ctx, gde_graph* G, int32_t* h_indices, int64_t* h_degree,
                               const int32_t* us, const int32_t* vs, int64_t k, int only_insert,
                               const gde_params* p, int64_t F, void* Pm, void* Rm, const void* Xm, int64_t ld,
                               double eps, double* oper_out, gde_stats* stats, uint8_t* outcome, bool edit_only) {
    const auto t_entry = std::chrono::steady_clock::now();
    auto since_entry = [&]() {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_entry).count();
    };
    if (!ctx || !G || !p || !h_indices || !h_degree || (k > 0 && (!us || !vs)))
        return gde_internal_fail(ctx, GDE_EINVAL, "bad update arguments");
    const int kind = p->kind;
    if (kind != KIND_IGN && kind != KIND_UPPR) return gde_internal_fail(ctx, GDE_EINVAL, "kind must be IGN or UPPR");
    if (kind == KIND_IGN && !Xm && !edit_only) return gde_internal_fail(ctx, GDE_EINVAL, "InstantGNN repair needs X");
    if (outcome && k > 0) memset(outcome, MIX_NOOP, (size_t)k);
    if (gde_internal_relabeled(G))
        return gde_internal_fail(ctx, GDE_EINVAL, "edge updates need a padded CSR graph (upload with row_len)");
    const int64_t* indptr;
    const int64_t* hlen;
    int64_t n;
    gde_internal_graph_host(G, &indptr, &hlen, &n);
    for (int64_t u = 0; u < n; u++)
        if (h_degree[u] != hlen[u])
            return gde_internal_fail(ctx, GDE_EINVAL, "host degree array differs from the resident graph");
    if (k > 0) {
        G->ncolors = 0;  // the edges change: the SOR colouring is rebuilt on its next use,
        G->dmax = -1.0;  // the degree bound recomputed and the spectral estimate dropped
        G->lam_max_est = NAN;
    }
    // ---- the edit, the repair keys and the push, all on the device ----
    if (k >= ((int64_t)1 << 30)) return gde_internal_fail(ctx, GDE_EINVAL, "edge batch too large (2^30 edges at most)");
    bool loops = false;
    for (int64_t e = 0; e < k; e++) {
        if (us[e] < 0 || us[e] >= n || vs[e] < 0 || vs[e] >= n)
            return gde_internal_fail(ctx, GDE_EINVAL, "edge endpoint out of range");
        loops = loops || us[e] == vs[e];
    }
    // The reference keeps one degree array that is both the row length and
    // the degree of the thresholds; an edit sets both from the new row.
    if (k > 0 && !G->deg_is_len)
        return gde_internal_fail(ctx, GDE_EINVAL, "edge batches need a padded graph whose degree is its row length");
    if (k == 0) {
        if (oper_out)
            for (int64_t c = 0; c < F; c++) oper_out[c] = 0.0;
        if (stats) {
            memset(stats, 0, sizeof(*stats));
            stats->edit_path = only_insert ? GDE_EDIT_DEVICE_INSERT : GDE_EDIT_DEVICE_DATAFLOW;
            stats->edit_ms = since_entry();
        }
        return GDE_OK;
    }
    if (kind == KIND_IGN) {
        int rc0 = gde_internal_ign_tables(ctx, G, p->beta);
        if (rc0 == GDE_OK) rc0 = ensure_power_tables(ctx, G, p->beta);
        if (rc0 != GDE_OK) return rc0;
    }
    // Insert-only batches decide every edge in parallel (device_insert); a
    // batch with deletions or self-loops, or an insert-only batch that finds
    // a row full, runs as the dataflow over the edges.
    DeviceEdit D;
    int path = GDE_EDIT_DEVICE_DATAFLOW;
    if (only_insert && !loops) {
        D = device_insert(ctx, G, h_indices, h_degree, us, vs, k, kind, p->beta, outcome);
        path = GDE_EDIT_DEVICE_INSERT;
    }
    if (path == GDE_EDIT_DEVICE_DATAFLOW || (D.status == GDE_OK && D.fallback)) {
        D = device_mixed_edit(ctx, G, h_indices, h_degree, us, vs, k, only_insert, kind, p->beta, outcome);
        path = GDE_EDIT_DEVICE_DATAFLOW;
    }
    if (D.status != GDE_OK) return D.status;
    // InstantGNN tables built for an earlier call are not updated by this
    // kind's edit: the next InstantGNN call rebuilds them
    if (kind != KIND_IGN) G->ign_beta = NAN;
    if (D.late_status != GDE_OK || edit_only) {
        // (a failing edge: the edges before it are applied, on the device and
        // in the caller's arrays, and nothing is repaired or pushed)
        if (stats) {
            memset(stats, 0, sizeof(*stats));
            stats->edit_path = path;
            stats->edit_ms = since_entry();
        }
        return D.late_status != GDE_OK ? gde_internal_fail(ctx, D.late_status, D.late_msg) : GDE_OK;
    }
    cudaStream_t st = gde_internal_stream(ctx);
    const int prec64 = (p->prec == GDE_FP64);
    if (D.nkeys > 0) {
        const int64_t total = (int64_t)D.nkeys * F;
        const int blocks = (int)((total + 255) / 256);
        if (prec64) {
            repair_pass1<double><<<blocks, 256, 0, st>>>(D.rkeys, D.nkeys, (double*)Pm, (double*)Rm, ld, F, kind,
                                                          p->alpha);
            repair_pass2<double><<<blocks, 256, 0, st>>>(D.rkeys, D.nkeys, D.nbr, (const double*)Pm, (double*)Rm,
                                                          (const double*)Xm, ld, F, kind, p->alpha,
                                                          gde_internal_npush(G), gde_internal_degd(G));
        } else {
            repair_pass1<float><<<blocks, 256, 0, st>>>(D.rkeys, D.nkeys, (float*)Pm, (float*)Rm, ld, F, kind,
                                                         p->alpha);
            repair_pass2<float><<<blocks, 256, 0, st>>>(D.rkeys, D.nkeys, D.nbr, (const float*)Pm, (float*)Rm,
                                                         (const float*)Xm, ld, F, kind, p->alpha,
                                                         gde_internal_npush(G), gde_internal_degd(G));
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return gde_internal_fail(ctx, GDE_ECUDA, cudaGetErrorString(e));
    }
    // ---- push from the repaired nodes (InstantGNN.py:315-325) ----
    std::vector<double> opers(F, 0.0);
    const double edit_ms = since_entry();
    if (D.nkeys > 0) {
        int rc = gde_internal_feature_push(ctx, G, p, F, Pm, Rm, ld, eps, D.keys, D.nkeys, opers.data(), stats);
        if (rc != GDE_OK) return rc;
    } else if (stats) {
        memset(stats, 0, sizeof(*stats));
    }
    // the beta = 0 PPR update counts the repair work (ppr_solver.py:776-792)
    const double oper_repair = 2.0 * (double)D.nkeys + (double)D.repair_nbr;
    if (oper_out)
        for (int64_t c = 0; c < F; c++) oper_out[c] = opers[c] + (kind == KIND_UPPR ? oper_repair : 0.0);
    if (stats) {
        stats->edit_path = path;
        stats->edit_ms = edit_ms;
    }
    return GDE_OK;
}

extern "C" int gde_feature_update(gde_ctx* ctx, gde_graph* G, int32_t* h_indices, int64_t* h_degree,
                                  const int32_t* us, const int32_t* vs, int64_t k, int only_insert,
                                  const gde_params* p, int64_t F, void* Pm, void* Rm, const void* Xm, int64_t ld,
                                  double eps, double* oper_out, gde_stats* stats) {
    return feature_update_impl(ctx, G, h_indices, h_degree, us, vs, k, only_insert, p, F, Pm, Rm, Xm, ld, eps,
                               oper_out, stats, nullptr, false);
}

extern "C" int gde_graph_update(gde_ctx* ctx, gde_graph* G, int32_t* h_indices, int64_t* h_degree, const int32_t* us,
                                const int32_t* vs, int64_t k, int only_insert, uint8_t* outcome, gde_stats* stats) {
    gde_params p;
    memset(&p, 0, sizeof p);
    p.kind = KIND_UPPR;  // no feature tables to keep up to date
    p.prec = GDE_FP64;
    return feature_update_impl(ctx, G, h_indices, h_degree, us, vs, k, only_insert, &p, 0, nullptr, nullptr, nullptr,
                               0, 0.0, nullptr, stats, outcome, true);
}

extern "C" int gde_feature_repair(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t F, void* Pm, void* Rm,
                                  const void* Xm, int64_t ld, int64_t nkeys, const int32_t* keys,
                                  const int64_t* old_degree, const int64_t* nbr_off, const int32_t* nbr) {
    if (!ctx || !G || !p || F < 0 || nkeys < 0 || (nkeys > 0 && (!keys || !old_degree || !nbr_off)))
        return gde_internal_fail(ctx, GDE_EINVAL, "bad repair arguments");
    const int kind = p->kind;
    if (kind != KIND_IGN && kind != KIND_UPPR) return gde_internal_fail(ctx, GDE_EINVAL, "kind must be IGN or UPPR");
    if (kind == KIND_IGN && !Xm) return gde_internal_fail(ctx, GDE_EINVAL, "InstantGNN repair needs X");
    if (nkeys == 0 || F == 0) return GDE_OK;
    if (nkeys >= ((int64_t)1 << 31) || nbr_off[2 * nkeys] >= ((int64_t)1 << 31))
        return gde_internal_fail(ctx, GDE_EINVAL, "repair lists too long");
    const int64_t* indptr;
    const int64_t* hlen;
    int64_t n;
    gde_internal_graph_host(G, &indptr, &hlen, &n);
    if (kind == KIND_IGN) {
        int rc0 = gde_internal_ign_tables(ctx, G, p->beta);
        if (rc0 != GDE_OK) return rc0;
    }
    // factors in the reference's operation order (InstantGNN.py:303-314,
    // ppr_solver.py:776-792), degrees after the batch from the resident graph
    std::vector<RepairKey> rk((size_t)nkeys);
    for (int64_t i = 0; i < nkeys; i++) {
        const int32_t u = keys[i];
        if (u < 0 || u >= n || !(old_degree[i] > 0)) return gde_internal_fail(ctx, GDE_EINVAL, "bad repair key");
        RepairKey& K = rk[(size_t)i];
        memset(&K, 0, sizeof K);
        K.u = u;
        const double d = (double)hlen[u], od = (double)old_degree[i];
        if (kind == KIND_IGN) {
            const double b = p->beta;
            K.a1 = std::pow(d / od, 1 - b);
            K.a2 = std::pow(od, 1 - b);
            K.a3 = std::pow(d, 1 - b);
            K.b1 = std::pow(od, b);
            K.b2 = std::pow(d, b);
        } else {
            K.a1 = d;
            K.a2 = od;
        }
        K.ins_beg = (int32_t)nbr_off[2 * i];
        K.ins_end = (int32_t)nbr_off[2 * i + 1];
        K.del_beg = K.ins_end;
        K.del_end = (int32_t)nbr_off[2 * i + 2];
    }
    const int64_t total = nbr_off[2 * nkeys];
    for (int64_t j = 0; j < total; j++)
        if (nbr[j] < 0 || nbr[j] >= n) return gde_internal_fail(ctx, GDE_EINVAL, "repair neighbour out of range");
    cudaStream_t st = gde_internal_stream(ctx);
    RepairKey* d_keys = (RepairKey*)gde_internal_wsget(ctx, "repair_keys", rk.size() * sizeof(RepairKey));
    int32_t* d_nbr = (int32_t*)gde_internal_wsget(ctx, "repair_nbr", (size_t)std::max<int64_t>(total, 1) * 4);
    if (!d_keys || !d_nbr) return gde_internal_fail(ctx, GDE_ENOMEM, "repair tables");
    if (cudaMemcpyAsync(d_keys, rk.data(), rk.size() * sizeof(RepairKey), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        (total > 0 && cudaMemcpyAsync(d_nbr, nbr, (size_t)total * 4, cudaMemcpyHostToDevice, st) != cudaSuccess))
        return gde_internal_fail(ctx, GDE_ECUDA, "repair upload");
    const int blocks = (int)((nkeys * F + 255) / 256);
    if (p->prec == GDE_FP64) {
        repair_pass1<double><<<blocks, 256, 0, st>>>(d_keys, (int)nkeys, (double*)Pm, (double*)Rm, ld, F, kind,
                                                      p->alpha);
        repair_pass2<double><<<blocks, 256, 0, st>>>(d_keys, (int)nkeys, d_nbr, (const double*)Pm, (double*)Rm,
                                                      (const double*)Xm, ld, F, kind, p->alpha,
                                                      gde_internal_npush(G), gde_internal_degd(G));
    } else {
        repair_pass1<float><<<blocks, 256, 0, st>>>(d_keys, (int)nkeys, (float*)Pm, (float*)Rm, ld, F, kind,
                                                     p->alpha);
        repair_pass2<float><<<blocks, 256, 0, st>>>(d_keys, (int)nkeys, d_nbr, (const float*)Pm, (float*)Rm,
                                                     (const float*)Xm, ld, F, kind, p->alpha, gde_internal_npush(G),
                                                     gde_internal_degd(G));
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return gde_internal_fail(ctx, GDE_ECUDA, cudaGetErrorString(e));
    return GDE_OK;
}
