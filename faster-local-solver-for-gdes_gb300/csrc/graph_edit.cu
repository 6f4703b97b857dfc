// graph_edit.cu -- dynamic padded-CSR edits and the incremental feature update.
//
// gde_feature_update = (1) apply an edge batch to the padded CSR with the
// sequential semantics of updetaGraph (InstantGNN.py:137-180, identical to
// updeta_graph at ppr_solver.py:723-766), mutating the caller's host arrays
// and the resident device graph; (2) repair P, R at the touched nodes on the
// GPU (InstantGNN.py:303-318 for InstantGNN, ppr_solver.py:776-792 for the
// beta = 0 PPR update); (3) push from the repaired nodes with the engine.
//
// The edit itself is a short sequential pass on the host (O(sum of scanned
// row lengths)); its effect on the device graph is uploaded as a list of
// (position, value) entries plus the new degree tables.
#include <cuda_runtime.h>

#include <cmath>
#include <algorithm>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "gde_common.cuh"
#include "gde_engine.h"

using namespace gde;

// Implemented in gde_capi.cu (shared internals).
int gde_internal_feature_push(gde_ctx* ctx, gde_graph* G, const gde_params* p, int64_t F, void* Pm, void* Rm,
                              int64_t ld, double eps, const int32_t* d_cand, int64_t ncand, double* oper_out,
                              gde_stats* stats);
int gde_internal_graph_refresh(gde_ctx* ctx, gde_graph* G, const int64_t* h_degree, const int64_t* pos,
                               const int32_t* val, int64_t nchg, double beta, int ign);
int gde_internal_graph_host(gde_graph* G, const int64_t** indptr, const int64_t** len, int64_t* n);
void* gde_internal_wsget(gde_ctx* ctx, const char* name, size_t bytes);
int gde_internal_fail(gde_ctx* ctx, int code, const char* msg);
cudaStream_t gde_internal_stream(gde_ctx* ctx);
const double* gde_internal_npush(gde_graph* G);
const double* gde_internal_degd(gde_graph* G);
bool gde_internal_relabeled(gde_graph* G);

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
    std::vector<int64_t> old_degree(h_degree, h_degree + n);
    // ---- (1) sequential edit, InstantGNN.py:147-179 ----
    KeyMap ins, del;
    std::vector<int64_t> pos;
    std::vector<int32_t> val;
    int status = GDE_OK;
    for (int64_t e = 0; e < k; e++) {
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
    int rc = gde_internal_graph_refresh(ctx, G, h_degree, pos.data(), val.data(), (int64_t)pos.size(), p->beta,
                                        kind == KIND_IGN);
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
    return GDE_OK;
}
