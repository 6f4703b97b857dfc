// graph_edit.cu -- dynamic padded-CSR edits and the incremental feature update.
//
// gde_feature_update = (1) apply an edge batch to the padded CSR with the
// sequential semantics of updetaGraph (InstantGNN.py:137-180, identical to
// updeta_graph at ppr_solver.py:723-766), mutating the caller's host arrays
// and the resident device graph; (2) repair P, R at the touched nodes on the
// GPU (InstantGNN.py:303-318 for InstantGNN, ppr_solver.py:776-792 for the
// beta = 0 PPR update); (3) push from the repaired nodes with the engine.
//
// Insert-only batches without self-loops are applied on the device
// (device_insert below): which edges are inserted and where every new entry
// lands are decided in parallel with exactly the sequential semantics, and
// the caller's host arrays receive the same values afterwards.  Deletions
// keep a short sequential pass on the host (O(sum of scanned row lengths)),
// whose effect on the device graph is uploaded as (position, value) entries
// plus the new degree tables.
#include <cuda_runtime.h>

#include <cmath>
#include <algorithm>
#include <cstring>
#include <string>
#include <unordered_map>
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

namespace {

struct KeyMap {
    std::vector<int64_t> keys;             // first-insertion order
    std::vector<std::vector<int64_t>> nbr; // appended neighbours
    std::unordered_map<int64_t, int64_t> slot;
    void add(int64_t a, int64_t b) {
        auto it = slot.find(a);
        int64_t s;
        if (it == slot.end()) {
            s = (int64_t)keys.size();
            slot.emplace(a, s);
            keys.push_back(a);
            nbr.emplace_back();
        } else {
            s = it->second;
        }
        nbr[s].push_back(b);
    }
};

// Per-key repair factors (computed on the host with the C library's pow,
// in the reference's operation order).
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
__global__ void ins_repair_keys_kernel(const int32_t* keys, int nkeys, const int* cnt, const int* off,
                                       const int32_t* row_len, int kind, double beta, const double* pw1,
                                       const double* pwb, RepairKey* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nkeys; i += gridDim.x * blockDim.x) {
        const int u = keys[i];
        const int d = row_len[u];
        const int od = d - cnt[u];
        RepairKey K;
        K.u = u;
        K.ins_beg = off[u];
        K.ins_end = off[u] + cnt[u];
        K.del_beg = K.del_end = K.ins_end;
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
// commute, so the batch runs as a dataflow: an edge executes once every
// earlier edge on both of its endpoints has, which reproduces the
// sequential result exactly.  Each node keeps the position of its next edge
// (`next`); every round a warp per ready edge scans the row, edits both rows
// and advances its endpoints; the earliest pending edge is always ready, so
// a batch of k edges ends within k rounds.
// ---------------------------------------------------------------------------
struct MixOp {
    int32_t u, v;    // endpoints (caller ids of the padded graph)
    int32_t tu, tv;  // their touched-node indices
    int32_t pu, pv;  // this edge's position in each endpoint's edge list
};

enum : uint8_t { MIX_NOOP = 0, MIX_INSERT = 1, MIX_DELETE = 2 };

__global__ void mix_edit_kernel(const int64_t* row_ptr, int32_t* col, int32_t* row_len, const MixOp* ops, int k,
                                int* next, uint8_t* done, uint8_t* outcome, int* ndone, GridBarrier* bar, int* err) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int round = 0; round <= k; ++round) {
        for (int e = warp; e < k; e += nwarps) {
            const MixOp op = ops[e];
            int ready = 0;  // decided by lane 0 for the whole warp
            if (lane == 0)
                ready = !*(volatile uint8_t*)&done[e] && ld_volatile_i(&next[op.tu]) == op.pu &&
                        ld_volatile_i(&next[op.tv]) == op.pv;
            if (!__shfl_sync(0xffffffffu, ready, 0)) continue;
            __threadfence();  // the earlier edges' writes before this edge's reads
            const int64_t ru = row_ptr[op.u], rv = row_ptr[op.v];
            const int du = __ldcg(&row_len[op.u]), dv = __ldcg(&row_len[op.v]);
            // first position of v in u's row (InstantGNN.py:153-155)
            int found = -1;
            for (int i0 = 0; i0 < du && found < 0; i0 += 32) {
                const bool m = (i0 + lane < du) && __ldcg(&col[ru + i0 + lane]) == op.v;
                const unsigned b = __ballot_sync(0xffffffffu, m);
                if (b) found = i0 + __ffs(b) - 1;
            }
            uint8_t oc = MIX_NOOP;
            if (found >= 0) {
                if (du > 1 && dv > 1) {  // the degree-1 guard keeps the edge (:157-158)
                    // swap-with-last in u's row; every u in v's row takes v's last entry (:159-162)
                    const int32_t lastv = __ldcg(&col[rv + dv - 1]);
                    if (lane == 0) col[ru + found] = __ldcg(&col[ru + du - 1]);
                    for (int j = lane; j < dv; j += 32)
                        if (__ldcg(&col[rv + j]) == op.u) col[rv + j] = lastv;
                    if (lane == 0) {
                        row_len[op.u] = du - 1;
                        row_len[op.v] = dv - 1;
                    }
                    oc = MIX_DELETE;
                }
            } else {
                // append to both rows (:171-174); slack was checked on the host
                if (lane == 0) {
                    col[ru + du] = op.v;
                    col[rv + dv] = op.u;
                    row_len[op.u] = du + 1;
                    row_len[op.v] = dv + 1;
                }
                oc = MIX_INSERT;
            }
            __threadfence();  // every lane's edit visible before the endpoints move on
            __syncwarp();
            if (lane == 0) {
                outcome[e] = oc;
                __threadfence();
                next[op.tu] = op.pu + 1;
                next[op.tv] = op.pv + 1;
                done[e] = 1;
                atomicAdd(ndone, 1);
            }
            __syncwarp();
        }
        // every block reads the count between two barriers, before any edge of
        // the next round runs, so all of them leave in the same round
        if (!grid_barrier(bar, err)) return;
        const bool fin = ld_volatile_i(ndone) >= k;
        if (!grid_barrier(bar, err)) return;
        if (fin) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(err, 0, GDE_EHANG);
}

struct MixResult {
    int status = GDE_OK;
    bool fallback = false;         // not eligible (self-loop, no slack): the host pass runs instead
    std::vector<uint8_t> outcome;  // per edge: MIX_NOOP / MIX_INSERT / MIX_DELETE
};

MixResult device_mixed_edit(gde_ctx* ctx, gde_graph* G, int32_t* h_indices, int64_t* h_degree, const int32_t* us,
                            const int32_t* vs, int64_t k) {
    MixResult M;
    const int64_t n = G->g.n;
    const int64_t* indptr;
    const int64_t* hlen;
    int64_t nn;
    gde_internal_graph_host(G, &indptr, &hlen, &nn);
    if (k >= ((int64_t)1 << 30)) { M.fallback = true; return M; }
    // touched nodes, and each edge's position in its endpoints' edge lists
    std::unordered_map<int32_t, int32_t> tix;
    tix.reserve((size_t)(2 * k));
    std::vector<int32_t> cnt;
    std::vector<MixOp> ops((size_t)k);
    for (int64_t e = 0; e < k; e++) {
        const int32_t u = us[e], v = vs[e];
        if (u == v) { M.fallback = true; return M; }  // self-loops keep the host pass
        auto a = tix.emplace(u, (int32_t)cnt.size());
        if (a.second) cnt.push_back(0);
        auto b = tix.emplace(v, (int32_t)cnt.size());
        if (b.second) cnt.push_back(0);
        MixOp& op = ops[(size_t)e];
        op.u = u; op.v = v;
        op.tu = a.first->second; op.tv = b.first->second;
        op.pu = cnt[op.tu]++;
        op.pv = cnt[op.tv]++;
    }
    // slack: a node gains at most one entry per edge touching it
    for (const auto& kv : tix)
        if (h_degree[kv.first] + cnt[kv.second] > indptr[kv.first + 1] - indptr[kv.first]) {
            M.fallback = true;
            return M;
        }
    const int64_t T = (int64_t)cnt.size();
    cudaStream_t st = ctx->stream;
    auto ws = [&](const char* name, size_t bytes) { return gde_internal_wsget(ctx, name, std::max<size_t>(bytes, 8)); };
    MixOp* d_ops = (MixOp*)ws("mix_ops", (size_t)k * sizeof(MixOp));
    int* d_next = (int*)ws("mix_next", (size_t)T * 4);
    uint8_t* d_done = (uint8_t*)ws("mix_done", (size_t)k);
    uint8_t* d_out = (uint8_t*)ws("mix_out", (size_t)k);
    int* d_ndone = (int*)ws("mix_ndone", 4);
    if (!d_ops || !d_next || !d_done || !d_out || !d_ndone) {
        M.status = gde_internal_fail(ctx, GDE_ENOMEM, "edit batch buffers");
        return M;
    }
    auto ck = [&](cudaError_t e2, const char* what) {
        if (e2 != cudaSuccess && M.status == GDE_OK) M.status = gde_internal_fail(ctx, GDE_ECUDA, what);
    };
    ck(cudaMemcpyAsync(d_ops, ops.data(), (size_t)k * sizeof(MixOp), cudaMemcpyHostToDevice, st), "edit upload");
    ck(cudaMemsetAsync(d_next, 0, (size_t)T * 4, st), "edit init");
    ck(cudaMemsetAsync(d_done, 0, (size_t)k, st), "edit init");
    ck(cudaMemsetAsync(d_ndone, 0, 4, st), "edit init");
    ck(cudaMemsetAsync(ctx->bar, 0, sizeof(GridBarrier), st), "edit init");
    ck(cudaMemsetAsync(ctx->derr, 0, sizeof(int), st), "edit init");
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mix_edit_kernel, kEdT, 0);
    const int64_t want = (k * 32 + kEdT - 1) / kEdT;  // a warp per edge at most
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::max(per_sm, 1) * ctx->sms, want));
    const int64_t* row_ptr = G->g.row_ptr;
    int32_t* col = G->col;
    int32_t* rl = G->row_len;
    int ki = (int)k;
    GridBarrier* bar = ctx->bar;
    int* err = ctx->derr;
    void* args[] = {(void*)&row_ptr, (void*)&col, (void*)&rl, (void*)&d_ops, (void*)&ki, (void*)&d_next,
                    (void*)&d_done, (void*)&d_out, (void*)&d_ndone, (void*)&bar, (void*)&err};
    if (M.status == GDE_OK)
        ck(cudaLaunchCooperativeKernel((void*)mix_edit_kernel, dim3(grid), dim3(kEdT), args, 0, st), "edit launch");
    int herr = 0;
    ck(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st), "edit status");
    ck(cudaStreamSynchronize(st), "edit kernel");
    if (M.status != GDE_OK) return M;
    if (herr != 0) {
        M.status = gde_internal_fail(ctx, GDE_EHANG, "edit batch: a device-side wait ran out");
        return M;
    }
    // the edited rows and degrees back into the caller's host arrays
    M.outcome.resize((size_t)k);
    std::vector<int32_t> len32((size_t)n);
    ck(cudaMemcpyAsync(M.outcome.data(), d_out, (size_t)k, cudaMemcpyDeviceToHost, st), "edit readback");
    ck(cudaMemcpyAsync(h_indices, col, (size_t)G->g.cap * 4, cudaMemcpyDeviceToHost, st), "edit readback");
    ck(cudaMemcpyAsync(len32.data(), rl, (size_t)n * 4, cudaMemcpyDeviceToHost, st), "edit readback");
    ck(cudaStreamSynchronize(st), "edit readback");
    if (M.status != GDE_OK) return M;
    for (const auto& kv : tix) h_degree[kv.first] = len32[(size_t)kv.first];
    return M;
}

struct DeviceInsert {
    int status = GDE_OK;
    bool fallback = false;       // capacity exceeded: the host pass reproduces the partial edit
    const int32_t* keys = nullptr;
    int nkeys = 0;
    RepairKey* rkeys = nullptr;
    const int32_t* nbr = nullptr;
    int64_t inserted = 0;
};

DeviceInsert device_insert(gde_ctx* ctx, gde_graph* G, int32_t* h_indices, int64_t* h_degree, const int32_t* us,
                           const int32_t* vs, int64_t k, int kind, double beta) {
    DeviceInsert R;
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
        // written yet; the host pass applies the sequential partial edit
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
        ins_repair_keys_kernel<<<(nkeys + kEdT - 1) / kEdT, kEdT, 0, st>>>(d_keys, nkeys, d_cnt, d_off, G->row_len,
                                                                          kind, beta, G->pw1, G->pwb, d_rk);
    DI_CK(cudaGetLastError());
    // ---- the same edit on the caller's host arrays and the host mirror ----
    std::vector<int64_t> hpos(total);
    std::vector<int32_t> hval(total);
    std::vector<int> hcnt(n);
    DI_CK(cudaMemcpyAsync(hpos.data(), d_pos, (size_t)total * 8, cudaMemcpyDeviceToHost, st));
    DI_CK(cudaMemcpyAsync(hval.data(), d_nbr, (size_t)total * 4, cudaMemcpyDeviceToHost, st));
    DI_CK(cudaMemcpyAsync(hcnt.data(), d_cnt, n * 4, cudaMemcpyDeviceToHost, st));
    DI_CK(cudaStreamSynchronize(st));
#undef DI_CK
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
    R.inserted = total / 2;
    return R;
}

}  // namespace

extern "C" int gde_feature_update(gde_ctx* ctx, gde_graph* G, int32_t* h_indices, int64_t* h_degree,
                                  const int32_t* us, const int32_t* vs, int64_t k, int only_insert,
                                  const gde_params* p, int64_t F, void* Pm, void* Rm, const void* Xm, int64_t ld,
                                  double eps, double* oper_out, gde_stats* stats) {
    if (!ctx || !G || !p || !h_indices || !h_degree || (k > 0 && (!us || !vs)))
        return gde_internal_fail(ctx, GDE_EINVAL, "bad update arguments");
    const int kind = p->kind;
    if (kind != KIND_IGN && kind != KIND_UPPR) return gde_internal_fail(ctx, GDE_EINVAL, "kind must be IGN or UPPR");
    if (kind == KIND_IGN && !Xm) return gde_internal_fail(ctx, GDE_EINVAL, "InstantGNN repair needs X");
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
    // ---- insert-only batches: the edit, the repair keys and the push all on the device ----
    bool dev_ok = only_insert && k > 0 && G->deg_is_len;
    for (int64_t e = 0; dev_ok && e < k; e++)
        dev_ok = us[e] >= 0 && us[e] < n && vs[e] >= 0 && vs[e] < n && us[e] != vs[e];
    if (dev_ok) {
        if (kind == KIND_IGN) {
            int rc0 = gde_internal_ign_tables(ctx, G, p->beta);
            if (rc0 == GDE_OK) rc0 = ensure_power_tables(ctx, G, p->beta);
            if (rc0 != GDE_OK) return rc0;
        }
        DeviceInsert D = device_insert(ctx, G, h_indices, h_degree, us, vs, k, kind, p->beta);
        if (D.status != GDE_OK) return D.status;
        // InstantGNN tables built for an earlier call are not updated by this
        // kind's edit: the next InstantGNN call rebuilds them
        if (kind != KIND_IGN) G->ign_beta = NAN;
        if (!D.fallback) {
            cudaStream_t st = gde_internal_stream(ctx);
            const int prec64 = (p->prec == GDE_FP64);
            if (D.nkeys > 0) {
                const int64_t total = (int64_t)D.nkeys * F;
                const int blocks = (int)((total + 255) / 256);
                if (prec64) {
                    repair_pass1<double><<<blocks, 256, 0, st>>>(D.rkeys, D.nkeys, (double*)Pm, (double*)Rm, ld, F,
                                                                  kind, p->alpha);
                    repair_pass2<double><<<blocks, 256, 0, st>>>(D.rkeys, D.nkeys, D.nbr, (const double*)Pm,
                                                                  (double*)Rm, (const double*)Xm, ld, F, kind,
                                                                  p->alpha, gde_internal_npush(G),
                                                                  gde_internal_degd(G));
                } else {
                    repair_pass1<float><<<blocks, 256, 0, st>>>(D.rkeys, D.nkeys, (float*)Pm, (float*)Rm, ld, F,
                                                                 kind, p->alpha);
                    repair_pass2<float><<<blocks, 256, 0, st>>>(D.rkeys, D.nkeys, D.nbr, (const float*)Pm,
                                                                 (float*)Rm, (const float*)Xm, ld, F, kind, p->alpha,
                                                                 gde_internal_npush(G), gde_internal_degd(G));
                }
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) return gde_internal_fail(ctx, GDE_ECUDA, cudaGetErrorString(e));
            }
            std::vector<double> opers(F, 0.0);
            if (D.nkeys > 0) {
                int rc = gde_internal_feature_push(ctx, G, p, F, Pm, Rm, ld, eps, D.keys, D.nkeys, opers.data(),
                                                   stats);
                if (rc != GDE_OK) return rc;
            } else if (stats) {
                memset(stats, 0, sizeof(*stats));
            }
            // the beta = 0 PPR update counts the repair work (ppr_solver.py:776-792)
            const double oper_repair = 2.0 * (double)D.nkeys + 2.0 * (double)D.inserted;
            if (oper_out)
                for (int64_t c = 0; c < F; c++) oper_out[c] = opers[c] + (kind == KIND_UPPR ? oper_repair : 0.0);
            if (stats) stats->edit_path = GDE_EDIT_DEVICE_INSERT;
            return GDE_OK;
        }
    }
    std::vector<int64_t> old_degree(h_degree, h_degree + n);
    // ---- (1) sequential edit, InstantGNN.py:147-179 ----
    KeyMap ins, del;
    std::vector<int64_t> pos;
    std::vector<int32_t> val;
    int status = GDE_OK;
    // batches with deletions run as a dataflow on the device (device_mixed_edit);
    // each edge's outcome there rebuilds the reference's insert / delete maps
    bool on_device = false;
    if (!only_insert && k > 0 && G->deg_is_len) {
        bool ok = true;
        for (int64_t e = 0; ok && e < k; e++) ok = us[e] >= 0 && us[e] < n && vs[e] >= 0 && vs[e] < n;
        if (ok) {
            MixResult M = device_mixed_edit(ctx, G, h_indices, h_degree, us, vs, k);
            if (M.status != GDE_OK) return M.status;
            if (!M.fallback) {
                on_device = true;
                for (int64_t e = 0; e < k; e++) {
                    if (M.outcome[(size_t)e] == MIX_INSERT) {
                        ins.add(us[e], vs[e]);
                        ins.add(vs[e], us[e]);
                    } else if (M.outcome[(size_t)e] == MIX_DELETE) {
                        del.add(us[e], vs[e]);
                        del.add(vs[e], us[e]);
                    }
                }
            }
        }
    }
    for (int64_t e = 0; e < k && !on_device; e++) {
        int64_t u = us[e], v = vs[e];
        if (u < 0 || u >= n || v < 0 || v >= n) { status = GDE_EINVAL; break; }
        bool insertion = true;
        for (int64_t i = indptr[u]; i < indptr[u] + h_degree[u]; i++) {
            if (v == h_indices[i]) {
                insertion = false;
                if (only_insert || h_degree[u] == 1 || h_degree[v] == 1) break;
                int64_t lu = indptr[u] + h_degree[u] - 1;
                h_indices[i] = h_indices[lu];
                pos.push_back(i); val.push_back(h_indices[i]);
                for (int64_t kk = indptr[v]; kk < indptr[v] + h_degree[v]; kk++)
                    if (u == h_indices[kk]) {
                        h_indices[kk] = h_indices[indptr[v] + h_degree[v] - 1];
                        pos.push_back(kk); val.push_back(h_indices[kk]);
                    }
                h_degree[u] -= 1;
                h_degree[v] -= 1;
                del.add(u, v);
                del.add(v, u);
                break;
            }
        }
        if (insertion) {
            if (indptr[u] + h_degree[u] >= indptr[u + 1] || indptr[v] + h_degree[v] >= indptr[v + 1] ||
                (u == v && indptr[u] + h_degree[u] + 1 >= indptr[u + 1])) {
                status = GDE_ECAPACITY;
                break;
            }
            int64_t pu = indptr[u] + h_degree[u], pv = indptr[v] + h_degree[v];
            h_indices[pu] = (int32_t)v;
            pos.push_back(pu); val.push_back((int32_t)v);
            h_indices[pv] = (int32_t)u;
            pos.push_back(pv); val.push_back((int32_t)u);
            h_degree[u] += 1;
            h_degree[v] += 1;
            ins.add(u, v);
            ins.add(v, u);
        }
    }
    // A slot can be written more than once (swap-with-last deletions); the
    // device receives each touched slot once, with its final value.
    std::sort(pos.begin(), pos.end());
    pos.erase(std::unique(pos.begin(), pos.end()), pos.end());
    val.resize(pos.size());
    for (size_t i = 0; i < pos.size(); i++) val[i] = h_indices[pos[i]];
    // only the nodes whose degree changed get new degree tables
    std::vector<int64_t> touched;
    touched.reserve(ins.keys.size() + del.keys.size());
    for (int64_t u : ins.keys) touched.push_back(u);
    for (int64_t u : del.keys) touched.push_back(u);
    std::sort(touched.begin(), touched.end());
    touched.erase(std::unique(touched.begin(), touched.end()), touched.end());
    int rc = gde_internal_graph_refresh_nodes(ctx, G, h_degree, touched.data(), (int64_t)touched.size(), pos.data(),
                                              val.data(), (int64_t)pos.size(), p->beta, kind == KIND_IGN);
    if (rc != GDE_OK) return rc;
    if (status != GDE_OK)
        return gde_internal_fail(ctx, status, status == GDE_ECAPACITY ? "padded row has no slack for an insertion"
                                                                      : "edge endpoint out of range");
    // ---- (2) repair at the touched nodes ----
    std::vector<RepairKey> keys;
    std::vector<int32_t> nbr;
    double oper_repair = 2.0 * (double)ins.keys.size();
    for (size_t s = 0; s < ins.keys.size(); s++) {
        RepairKey K{};
        int64_t u = ins.keys[s];
        K.u = (int32_t)u;
        double d = (double)h_degree[u], od = (double)old_degree[u];
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
        K.ins_beg = (int32_t)nbr.size();
        for (int64_t v : ins.nbr[s]) nbr.push_back((int32_t)v);
        K.ins_end = (int32_t)nbr.size();
        oper_repair += (double)ins.nbr[s].size();
        K.del_beg = K.del_end = K.ins_end;
        bool use_del = (kind == KIND_UPPR) || !only_insert;
        auto it = del.slot.find(u);
        if (use_del && it != del.slot.end()) {
            for (int64_t v : del.nbr[it->second]) nbr.push_back((int32_t)v);
            K.del_end = (int32_t)nbr.size();
            oper_repair += (double)del.nbr[it->second].size();
        }
        keys.push_back(K);
    }
    cudaStream_t st = gde_internal_stream(ctx);
    const int prec64 = (p->prec == GDE_FP64);
    std::vector<int32_t> cand;
    if (!keys.empty()) {
        RepairKey* d_keys = (RepairKey*)gde_internal_wsget(ctx, "repair_keys", keys.size() * sizeof(RepairKey));
        int32_t* d_nbr = (int32_t*)gde_internal_wsget(ctx, "repair_nbr", std::max<size_t>(nbr.size(), 1) * 4);
        if (!d_keys || !d_nbr) return gde_internal_fail(ctx, GDE_ENOMEM, "repair tables");
        cudaMemcpyAsync(d_keys, keys.data(), keys.size() * sizeof(RepairKey), cudaMemcpyHostToDevice, st);
        if (!nbr.empty()) cudaMemcpyAsync(d_nbr, nbr.data(), nbr.size() * 4, cudaMemcpyHostToDevice, st);
        int64_t total = (int64_t)keys.size() * F;
        int blocks = (int)((total + 255) / 256);
        if (prec64) {
            repair_pass1<double><<<blocks, 256, 0, st>>>(d_keys, (int)keys.size(), (double*)Pm, (double*)Rm, ld, F,
                                                          kind, p->alpha);
            repair_pass2<double><<<blocks, 256, 0, st>>>(d_keys, (int)keys.size(), d_nbr, (const double*)Pm,
                                                          (double*)Rm, (const double*)Xm, ld, F, kind, p->alpha,
                                                          gde_internal_npush(G), gde_internal_degd(G));
        } else {
            repair_pass1<float><<<blocks, 256, 0, st>>>(d_keys, (int)keys.size(), (float*)Pm, (float*)Rm, ld, F, kind,
                                                         p->alpha);
            repair_pass2<float><<<blocks, 256, 0, st>>>(d_keys, (int)keys.size(), d_nbr, (const float*)Pm, (float*)Rm,
                                                         (const float*)Xm, ld, F, kind, p->alpha,
                                                         gde_internal_npush(G), gde_internal_degd(G));
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return gde_internal_fail(ctx, GDE_ECUDA, cudaGetErrorString(e));
        for (auto& K : keys) cand.push_back(K.u);
    }
    // ---- (3) push from the repaired nodes (InstantGNN.py:315-325) ----
    std::vector<double> opers(F, 0.0);
    if (!cand.empty()) {
        int32_t* d_cand = (int32_t*)gde_internal_wsget(ctx, "update_cand", cand.size() * 4);
        if (!d_cand) return gde_internal_fail(ctx, GDE_ENOMEM, "candidate list");
        cudaMemcpyAsync(d_cand, cand.data(), cand.size() * 4, cudaMemcpyHostToDevice, st);
        rc = gde_internal_feature_push(ctx, G, p, F, Pm, Rm, ld, eps, d_cand, (int64_t)cand.size(), opers.data(),
                                       stats);
        if (rc != GDE_OK) return rc;
    } else if (stats) {
        memset(stats, 0, sizeof(*stats));
    }
    if (oper_out)
        for (int64_t c = 0; c < F; c++) oper_out[c] = opers[c] + (kind == KIND_UPPR ? oper_repair : 0.0);
    if (stats) stats->edit_path = on_device ? GDE_EDIT_DEVICE_DATAFLOW : GDE_EDIT_HOST;
    return GDE_OK;
}
