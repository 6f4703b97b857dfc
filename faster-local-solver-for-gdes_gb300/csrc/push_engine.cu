// push_engine.cu -- persistent synchronous local-push kernel for sm_103a.
//
// One cooperative launch advances every live tile through up to
// `round_budget` push rounds.  A round is two phases separated by a bounded
// grid barrier (global GD/Chebyshev tiles add a CHECK phase in front):
//
//   PREP    (per tile) visit the candidates (the nodes touched last round, or
//           every node when the frontier was dense), test |r| >= threshold per
//           column in FP64, move the active residual into the solution
//           (Kahan-compensated in FP32), compute the push row P[f][0..W), and
//           compact the union frontier with a warp ballot + block prefix sum +
//           one global atomic per block, bucketed by degree.
//   SCATTER (per tile) push P rows along the CSR rows: long rows in CTA-sized
//           chunks, medium rows one warp per row, short rows one lane group
//           per row; W columns move per edge with one vector atomic; touched
//           nodes are appended (deduplicated by a round stamp) as the next
//           round's candidates unless the next round scans densely.
//
// Semantics follow the reference's synchronous round of ppr_gd local
// (ppr_solver.py:246-288): the frontier of round t+1 is exactly the set of
// nodes whose residual passes eps_vec after round t.
#include <cuda_runtime.h>

#include "gde_common.cuh"
#include "gde_device.cuh"
#include "gde_engine.h"

namespace gde {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr unsigned kFull = 0xffffffffu;
constexpr unsigned long long kSpinLimit = 1ull << 26;  // ~ seconds of polling

// ---------------------------------------------------------------------------
// Bounded grid barrier (sense by generation counter).  Co-residency of all
// blocks is guaranteed by the cooperative launch; the spin limit only guards
// against a bug turning into a hang: on expiry the block records GDE_EHANG
// and every block leaves its loop at the next barrier.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) { return *(volatile const unsigned*)p; }
__device__ __forceinline__ int ld_volatile_i(const int* p) { return *(volatile const int*)p; }

__device__ bool grid_barrier(GridBarrier* bar, int* err) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        unsigned gen = ld_volatile(&bar->gen);
        __threadfence();
        unsigned arrived = atomicAdd(&bar->count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            unsigned long long spins = 0;
            while (ld_volatile(&bar->gen) == gen) {
                if (ld_volatile_i(err) != 0) { ok = 0; break; }
                if (++spins > kSpinLimit) { atomicCAS(err, 0, GDE_EHANG); ok = 0; break; }
                __nanosleep(100);
            }
        }
        __threadfence();
        if (ld_volatile_i(err) != 0) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// ---------------------------------------------------------------------------
// Vector helpers: VEC contiguous columns per lane.
// ---------------------------------------------------------------------------
template <typename T, int VEC>
struct Vec {
    T v[VEC];
};

template <typename T, int VEC>
__device__ __forceinline__ void vload(const T* p, Vec<T, VEC>& o) {
#pragma unroll
    for (int i = 0; i < VEC; ++i) o.v[i] = p[i];
}
template <>
__device__ __forceinline__ void vload<float, 4>(const float* p, Vec<float, 4>& o) {
    float4 t = *reinterpret_cast<const float4*>(p);
    o.v[0] = t.x; o.v[1] = t.y; o.v[2] = t.z; o.v[3] = t.w;
}
template <>
__device__ __forceinline__ void vload<float, 2>(const float* p, Vec<float, 2>& o) {
    float2 t = *reinterpret_cast<const float2*>(p);
    o.v[0] = t.x; o.v[1] = t.y;
}
template <>
__device__ __forceinline__ void vload<double, 2>(const double* p, Vec<double, 2>& o) {
    double2 t = *reinterpret_cast<const double2*>(p);
    o.v[0] = t.x; o.v[1] = t.y;
}

template <typename T, int VEC>
__device__ __forceinline__ void vstore(T* p, const Vec<T, VEC>& o) {
#pragma unroll
    for (int i = 0; i < VEC; ++i) p[i] = o.v[i];
}
template <>
__device__ __forceinline__ void vstore<float, 4>(float* p, const Vec<float, 4>& o) {
    *reinterpret_cast<float4*>(p) = make_float4(o.v[0], o.v[1], o.v[2], o.v[3]);
}
template <>
__device__ __forceinline__ void vstore<float, 2>(float* p, const Vec<float, 2>& o) {
    *reinterpret_cast<float2*>(p) = make_float2(o.v[0], o.v[1]);
}
template <>
__device__ __forceinline__ void vstore<double, 2>(double* p, const Vec<double, 2>& o) {
    *reinterpret_cast<double2*>(p) = make_double2(o.v[0], o.v[1]);
}

// atomic add of VEC contiguous values, result unused (reduction)
template <typename T, int VEC>
__device__ __forceinline__ void vred(T* p, const Vec<T, VEC>& o) {
#pragma unroll
    for (int i = 0; i < VEC; ++i)
        if (o.v[i] != T(0)) atomicAdd(p + i, o.v[i]);
}
template <>
__device__ __forceinline__ void vred<float, 4>(float* p, const Vec<float, 4>& o) {
    atomicAdd(reinterpret_cast<float4*>(p), make_float4(o.v[0], o.v[1], o.v[2], o.v[3]));
}
template <>
__device__ __forceinline__ void vred<float, 2>(float* p, const Vec<float, 2>& o) {
    atomicAdd(reinterpret_cast<float2*>(p), make_float2(o.v[0], o.v[1]));
}

template <typename T>
__device__ __forceinline__ T* slab_ptr(void* base, const PushArgs& a, int t) {
    return reinterpret_cast<T*>(base) + (int64_t)t * a.tile_stride;
}

// Per-tile data staged in shared memory at the start of each tile's phase.
struct TileSh {
    TileParams tp;
    int cand_cnt, front_cnt, small_cnt, med_cnt, large_cnt;
    int dense, parity, level, stamp, m3;
    double psi;             // HK: psi[level]
    double coef1, coef2;    // Chebyshev coefficients of this round
    int final_level;        // HK: pushes of this level go into X
    int col_live[kMaxW];
    double col_theta[kMaxW];
};

constexpr int kMaxTiles = 4096;

__device__ __forceinline__ bool is_absorbing(const DevGraph& g, int u) {
    int len = g.row_len[u];
    return len == 0 || (len == 1 && g.col[g.row_ptr[u]] == u);
}

__device__ __forceinline__ bool hk_last_level(const TileSh& sh) {
    return (sh.tp.method == M_HK_TAYLOR) ? (sh.level >= sh.tp.n_levels) : (sh.level + 1 >= sh.tp.n_levels);
}

// Load the state of tile t at launch iteration `it` (block-wide).
template <int W>
__device__ void load_tile(const PushArgs& a, int t, int it, TileSh& sh) {
    if (threadIdx.x == 0) {
        const TileState& ts = a.ts[t];
        sh.tp = a.tp[t];
        sh.level = ts.round + it;
        int par = sh.level & 1;
        sh.parity = par;
        sh.m3 = sh.level % 3;
        sh.cand_cnt = ts.cand_cnt[sh.m3];
        sh.front_cnt = ts.front_cnt[par];
        sh.small_cnt = ts.small_cnt[par];
        sh.med_cnt = ts.med_cnt[par];
        sh.large_cnt = ts.large_cnt[par];
        sh.dense = ts.dense_next[par];
        sh.stamp = ts.stamp + sh.level + 1;
        int m = sh.tp.method;
        sh.psi = 1.0;
        sh.final_level = 0;
        if (method_is_hk(m)) {
            sh.psi = sh.tp.psi_tab[sh.level];
            sh.final_level = (m != M_HK_TAYLOR) && (sh.level + 1 == sh.tp.n_levels);
        }
        sh.coef1 = sh.coef2 = 0.0;
        if (method_is_cheby(m)) {
            if (sh.tp.kind == KIND_KATZ) {
                sh.coef1 = sh.tp.coef_tab[2 * sh.level];
                sh.coef2 = sh.tp.coef_tab[2 * sh.level + 1];
            } else {
                sh.coef1 = sh.tp.coef_tab[sh.level];
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < W) {
        const ColState& c = a.cs[(int64_t)t * W + threadIdx.x];
        int live = (threadIdx.x < sh.tp.ncols) && c.live;
        int m = sh.tp.method;
        // global GD / Chebyshev: a column whose CHECK found no node above
        // threshold stops before updating (ppr_solver.py:292-293)
        if (live && (m == M_GLOBAL_GD || m == M_GLOBAL_CHEBY) && c.check_cnt[sh.parity] == 0) live = 0;
        sh.col_theta[threadIdx.x] = c.theta;
        sh.col_live[threadIdx.x] = live;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// CHECK phase (global GD / Chebyshev): count per column the nodes with
// |r| >= eps_vec (ppr_solver.py:292, :605; katz_solver.py:227, :363).
// ---------------------------------------------------------------------------
template <typename T, int W>
__device__ void check_phase(const PushArgs& a, int t, int it, int* s_cnt) {
    constexpr int VEC = (sizeof(T) == 4) ? (W >= 4 ? 4 : W) : (W >= 2 ? 2 : 1);
    constexpr int L = W / VEC;
    __shared__ int s_live[kMaxW];
    __shared__ double s_theta[kMaxW];
    __shared__ int s_par;
    const int64_t n = a.g.n;
    const T* R = slab_ptr<T>(a.R, a, t);
    if (threadIdx.x == 0) s_par = (a.ts[t].round + it) & 1;
    if (threadIdx.x < W) {
        const ColState& c = a.cs[(int64_t)t * W + threadIdx.x];
        s_live[threadIdx.x] = (threadIdx.x < a.tp[t].ncols) && c.live;
        s_theta[threadIdx.x] = c.theta;
        s_cnt[threadIdx.x] = 0;
    }
    __syncthreads();
    int lane_g = threadIdx.x % L;
    int c0 = lane_g * VEC;
    int cnt[VEC];
#pragma unroll
    for (int i = 0; i < VEC; ++i) cnt[i] = 0;
    int64_t gid = ((int64_t)blockIdx.x * kThreads + threadIdx.x) / L;
    int64_t ng = (int64_t)gridDim.x * kThreads / L;
    for (int64_t u = gid; u < n; u += ng) {
        Vec<T, VEC> rv;
        vload<T, VEC>(R + u * a.ld + c0, rv);
        double d = a.g.degd[u];
#pragma unroll
        for (int i = 0; i < VEC; ++i) {
            double thr = s_theta[c0 + i] * d;
            cnt[i] += (s_live[c0 + i] && fabs((double)rv.v[i]) >= thr) ? 1 : 0;
        }
    }
#pragma unroll
    for (int i = 0; i < VEC; ++i)
        if (cnt[i]) atomicAdd(&s_cnt[c0 + i], cnt[i]);
    __syncthreads();
    if (threadIdx.x < W && s_cnt[threadIdx.x])
        atomicAdd(&a.cs[(int64_t)t * W + threadIdx.x].check_cnt[s_par], s_cnt[threadIdx.x]);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// PREP phase
// ---------------------------------------------------------------------------
struct PrepSh {
    int warp_cnt[kWarps][4];
    int base[4];
    double col_oper[kMaxW];
    int col_nodes[kMaxW];
    double vol;
    int nodes;
};

template <typename T, int W>
__device__ void prep_phase(const PushArgs& a, int t, TileSh& sh, PrepSh& ps) {
    constexpr int VEC = (sizeof(T) == 4) ? (W >= 4 ? 4 : W) : (W >= 2 ? 2 : 1);
    constexpr int L = W / VEC;          // lanes per node
    constexpr int GPW = 32 / L;         // nodes per warp iteration
    const DevGraph& g = a.g;
    const int64_t n = g.n;
    const int par = sh.parity;
    const int kind = sh.tp.kind, method = sh.tp.method;
    const bool global = method_is_global(method);
    const bool cheby = method_is_cheby(method);
    const bool hk = method_is_hk(method);
    const bool ign = (kind == KIND_IGN || kind == KIND_UPPR);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lane_g = threadIdx.x % L, grp_w = lane / L;
    const int c0 = lane_g * VEC;
    const int64_t ncand = sh.dense ? n : sh.cand_cnt;
    const int32_t* cand = a.cand + ((int64_t)t * 2 + par) * n;
    int32_t* next = a.cand + ((int64_t)t * 2 + (par ^ 1)) * n;
    int32_t* mark = a.mark + (int64_t)t * n;
    int32_t* front = a.front + (int64_t)t * n;
    T* Pw = reinterpret_cast<T*>(a.P) + (int64_t)t * n * W;
    int32_t* bsmall = a.bsmall + (int64_t)t * n;
    int32_t* bmed = a.bmed + (int64_t)t * n;
    int2* blarge = a.blarge + (int64_t)t * a.large_cap;
    TileState& ts = a.ts[t];
    T* R = slab_ptr<T>((hk && (sh.level & 1)) ? a.R2 : a.R, a, t);
    T* X = slab_ptr<T>(a.X, a, t);
    float* XC = a.kahan ? slab_ptr<float>(a.XC, a, t) : nullptr;
    T* DX = cheby ? slab_ptr<T>(a.DX, a, t) : nullptr;
    const double alpha = sh.tp.alpha;

    if (threadIdx.x < W) { ps.col_oper[threadIdx.x] = 0.0; ps.col_nodes[threadIdx.x] = 0; }
    if (threadIdx.x == 0) { ps.vol = 0.0; ps.nodes = 0; }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int np = par ^ 1;
        ts.cand_cnt[(sh.level + 2) % 3] = 0;
        ts.front_cnt[np] = 0;
        ts.small_cnt[np] = 0;
        ts.med_cnt[np] = 0;
        ts.large_cnt[np] = 0;
        ts.union_vol[np] = 0.0;
    }
    if (blockIdx.x == 0 && threadIdx.x < W) {
        a.cs[(int64_t)t * W + threadIdx.x].round_active[par ^ 1] = 0;
        a.cs[(int64_t)t * W + threadIdx.x].check_cnt[par ^ 1] = 0;
    }
    __syncthreads();

    double my_oper[VEC];
    int my_nodes[VEC];
#pragma unroll
    for (int i = 0; i < VEC; ++i) { my_oper[i] = 0.0; my_nodes[i] = 0; }
    double my_vol = 0.0;
    int my_cnt = 0;
    int* next_cnt = &ts.cand_cnt[(sh.level + 1) % 3];

    // Warps stride independently over the candidates; the starting warp is
    // rotated by tile so that short lists spread over SMs.
    const int64_t nwarps = (int64_t)gridDim.x * kWarps;
    const int64_t wstart = ((int64_t)blockIdx.x * kWarps + warp + (int64_t)t * 131) % nwarps;
    for (int64_t base = wstart * GPW; base < ncand; base += nwarps * GPW) {
        int64_t i = base + grp_w;
        bool valid = i < ncand;
        int u = 0;
        bool act[VEC];
        Vec<T, VEC> push;
#pragma unroll
        for (int k = 0; k < VEC; ++k) { act[k] = false; push.v[k] = T(0); }
        double du = 1.0;
        int len = 0;
        bool absorb = false;
        if (valid) {
            u = sh.dense ? (int)i : cand[i];
            du = g.degd[u];
            len = g.row_len[u];
            const int64_t off = (int64_t)u * a.ld + c0;
            Vec<T, VEC> r;
            vload<T, VEC>(R + off, r);
            const double thr_base = (kind == KIND_IGN) ? g.nfac[u] : du;
            absorb = ign && is_absorbing(g, u);
            Vec<T, VEC> dxv;
            if (cheby) vload<T, VEC>(DX + off, dxv);
            bool any_write = false;
            Vec<T, VEC> xadd;
#pragma unroll
            for (int k = 0; k < VEC; ++k) {
                xadd.v[k] = T(0);
                const int c = c0 + k;
                if (!sh.col_live[c]) continue;
                const double rv = (double)r.v[k];
                double thr;
                if (hk) thr = ((sh.col_theta[c] * thr_base) / (double)sh.tp.n_levels) / sh.psi;
                else thr = sh.col_theta[c] * thr_base;
                bool a_k;
                if (cheby) {
                    // ppr_solver.py:642-646 / katz_solver.py:407-411
                    double tmp;
                    if (kind == KIND_KATZ) tmp = sh.coef1 * rv - sh.coef2 * (double)dxv.v[k];
                    else tmp = sh.coef1 * rv + (sh.coef1 - 1.) * (double)dxv.v[k];
                    a_k = global ? (tmp != 0.0) : (fabs(rv) >= thr);
                    if (a_k) {
                        T tmpT = (T)tmp;
                        xadd.v[k] = tmpT;
                        dxv.v[k] = tmpT;
                        r.v[k] = (T)(rv - (double)tmpT);  // rt[u] += -delta_xt[u] (:657)
                        double pv = (kind == KIND_KATZ) ? alpha * (double)tmpT : ((1. - alpha) * (double)tmpT) / du;
                        push.v[k] = (T)pv;
                    }
                } else {
                    a_k = global ? (rv != 0.0) : (fabs(rv) >= thr);
                    // An absorbing node (threshold 0) is visited once by the
                    // reference's initial scan and never re-enqueued; with a
                    // zero residual it has nothing to absorb.
                    if (absorb && rv == 0.0) a_k = false;
                    if (a_k) {
                        double pv;
                        if (kind == KIND_PPR || kind == KIND_UPPR) pv = ((1. - alpha) * rv) / du;
                        else if (kind == KIND_KATZ) pv = alpha * rv;
                        else if (kind == KIND_HK) {
                            if (sh.final_level) pv = rv / du;  // hk_solver.py:254-256
                            else pv = ((sh.tp.tau / ((double)sh.level + 1.)) * rv) / du;
                        } else {
                            pv = ((1. - alpha) * rv) / g.npush[u];  // InstantGNN.py:28
                        }
                        if (absorb) pv = 0.0;
                        push.v[k] = (T)pv;
                        xadd.v[k] = (kind == KIND_IGN && !absorb) ? (T)(sh.tp.x_gain * rv) : r.v[k];
                        r.v[k] = T(0);
                    }
                }
                act[k] = a_k;
                if (a_k) {
                    any_write = true;
                    my_nodes[k] += 1;
                    if (!absorb) my_oper[k] += du;
                }
            }
            if (any_write) {
                vstore<T, VEC>(R + off, r);
                if (cheby) vstore<T, VEC>(DX + off, dxv);
                Vec<T, VEC> xv;
                vload<T, VEC>(X + off, xv);
                if (absorb) {
                    // p[u] = r[u]; r[u] = 0 for an absorbing node (InstantGNN.py:22-25)
#pragma unroll
                    for (int k = 0; k < VEC; ++k)
                        if (act[k]) {
                            xv.v[k] = xadd.v[k];
                            if (XC) XC[off + k] = 0.f;
                        }
                } else if (XC) {
                    // Kahan-compensated FP32 accumulation of the solution
#pragma unroll
                    for (int k = 0; k < VEC; ++k)
                        if (act[k]) {
                            float cc = XC[off + k];
                            float y = (float)xadd.v[k] - cc;
                            float s = (float)xv.v[k] + y;
                            XC[off + k] = (s - (float)xv.v[k]) - y;
                            xv.v[k] = (T)s;
                        }
                } else {
#pragma unroll
                    for (int k = 0; k < VEC; ++k)
                        if (act[k]) xv.v[k] = xv.v[k] + xadd.v[k];
                }
                vstore<T, VEC>(X + off, xv);
            }
        }
        // ---- node-level frontier decision (OR over the lane group) ----
        bool any = false;
#pragma unroll
        for (int k = 0; k < VEC; ++k) any |= act[k];
        unsigned bal = __ballot_sync(kFull, any);
        unsigned gmask = ((L == 32) ? kFull : ((1u << L) - 1u)) << (grp_w * L);
        bool node_act = valid && (bal & gmask) != 0;
        bool leader = (lane_g == 0);
        // Chebyshev moves r[u] by -dx[u]: u itself is a candidate next round
        if (cheby && !global) append_once(leader && node_act, u, mark, sh.stamp, next, next_cnt, kFull);
        bool node_in = node_act && !absorb;  // absorbed nodes do not push
        int nch = 0;
        int bucket = -1;  // 0 small, 1 medium, 2 large
        if (node_in) {
            if (len <= a.small_max) bucket = 0;
            else if (len <= a.med_max) bucket = 1;
            else { bucket = 2; nch = (len + a.chunk - 1) / a.chunk; }
        }
        unsigned bf = __ballot_sync(kFull, leader && node_in);
        unsigned bs = __ballot_sync(kFull, leader && bucket == 0);
        unsigned bm = __ballot_sync(kFull, leader && bucket == 1);
        int lch = (leader && bucket == 2) ? nch : 0;
        int sc = lch;  // inclusive warp scan of chunk counts
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(kFull, sc, o);
            if (lane >= o) sc += y;
        }
        int wch = __shfl_sync(kFull, sc, 31);
        // one global atomic per non-empty list per warp
        int b0 = 0, b1 = 0, b2 = 0, b3 = 0;
        if (lane == 0 && bf) {
            b0 = atomicAdd(&ts.front_cnt[par], __popc(bf));
            if (bs) b1 = atomicAdd(&ts.small_cnt[par], __popc(bs));
            if (bm) b2 = atomicAdd(&ts.med_cnt[par], __popc(bm));
            if (wch) b3 = atomicAdd(&ts.large_cnt[par], wch);
        }
        unsigned below = (1u << lane) - 1u;
        int fidx = 0;
        if (bf) {
            b0 = __shfl_sync(kFull, b0, 0);
            b1 = __shfl_sync(kFull, b1, 0);
            b2 = __shfl_sync(kFull, b2, 0);
            b3 = __shfl_sync(kFull, b3, 0);
            if (leader && node_in) {
                fidx = b0 + __popc(bf & below);
                front[fidx] = u;
                if (bucket == 0) bsmall[b1 + __popc(bs & below)] = fidx;
                else if (bucket == 1) bmed[b2 + __popc(bm & below)] = fidx;
                else {
                    int lb = b3 + (sc - lch);
                    for (int ch = 0; ch < nch; ++ch) blarge[lb + ch] = make_int2(fidx, ch);
                }
                my_vol += du;
                my_cnt += 1;
            }
            fidx = __shfl_sync(kFull, fidx, grp_w * L);
            if (node_in) vstore<T, VEC>(Pw + (int64_t)fidx * W + c0, push);
        }
    }
    // ---- flush per-column counters ----
#pragma unroll
    for (int k = 0; k < VEC; ++k) {
        if (my_nodes[k]) {
            atomicAdd(&ps.col_nodes[c0 + k], my_nodes[k]);
            atomicAdd(&ps.col_oper[c0 + k], my_oper[k]);
        }
    }
    if (my_cnt) {
        atomicAdd(&ps.vol, my_vol);
        atomicAdd(&ps.nodes, my_cnt);
    }
    __syncthreads();
    if (threadIdx.x < W && ps.col_nodes[threadIdx.x]) {
        ColState& cs = a.cs[(int64_t)t * W + threadIdx.x];
        atomicAdd(&cs.round_active[par], ps.col_nodes[threadIdx.x]);
        atomicAdd(&cs.oper, ps.col_oper[threadIdx.x]);
        atomicAdd((unsigned long long*)&cs.fsum, (unsigned long long)ps.col_nodes[threadIdx.x]);
        atomicAdd(&a.stats->col_nodes, (unsigned long long)ps.col_nodes[threadIdx.x]);
        atomicAdd(&a.stats->col_vol, ps.col_oper[threadIdx.x]);
    }
    if (threadIdx.x == 0 && ps.nodes) {
        atomicAdd(&ts.union_vol[par], ps.vol);
        atomicAdd(&a.stats->union_nodes, (unsigned long long)ps.nodes);
        atomicAdd(&a.stats->union_vol, ps.vol);
    }
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(&a.stats->cand_nodes, (unsigned long long)ncand);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// SCATTER phase
// ---------------------------------------------------------------------------
template <typename T, int VEC>
__device__ __forceinline__ void push_edge(const DevGraph& g, T* tgt, int64_t ld, int c0, int v, const Vec<T, VEC>& p,
                                          bool tgt_scale) {
    Vec<T, VEC> q = p;
    if (tgt_scale) {
        // InstantGNN divides by d_v^beta at the target (InstantGNN.py:31)
        T dv = (sizeof(T) == 4) ? (T)g.tfac_f[v] : (T)g.tfac[v];
#pragma unroll
        for (int i = 0; i < VEC; ++i) q.v[i] = q.v[i] / dv;
    }
    vred<T, VEC>(tgt + (int64_t)v * ld + c0, q);
}

template <typename T, int W>
__device__ void scatter_phase(const PushArgs& a, int t, TileSh& sh) {
    constexpr int VEC = (sizeof(T) == 4) ? (W >= 4 ? 4 : W) : (W >= 2 ? 2 : 1);
    constexpr int L = W / VEC;
    constexpr int GPW = 32 / L;
    const DevGraph& g = a.g;
    const int64_t n = g.n;
    const int par = sh.parity;
    const int kind = sh.tp.kind, method = sh.tp.method;
    const bool hk = method_is_hk(method);
    const bool global = method_is_global(method);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lane_g = threadIdx.x % L, grp_w = lane / L;
    const int c0 = lane_g * VEC;
    TileState& ts = a.ts[t];
    const int32_t* front = a.front + (int64_t)t * n;
    const T* Pw = reinterpret_cast<const T*>(a.P) + (int64_t)t * n * W;
    const int32_t* bsmall = a.bsmall + (int64_t)t * n;
    const int32_t* bmed = a.bmed + (int64_t)t * n;
    const int2* blarge = a.blarge + (int64_t)t * a.large_cap;
    int32_t* mark = a.mark + (int64_t)t * n;
    int32_t* next = a.cand + ((int64_t)t * 2 + (par ^ 1)) * n;
    int* next_cnt = &ts.cand_cnt[(sh.level + 1) % 3];
    T* Tgt;
    if (hk) {
        if (sh.final_level) Tgt = slab_ptr<T>(a.X, a, t);
        else Tgt = slab_ptr<T>((sh.level & 1) ? a.R : a.R2, a, t);
    } else {
        Tgt = slab_ptr<T>(a.R, a, t);
    }
    // Does the next round scan densely?  Every block decides identically.
    // Thresholds can drop between solves (a dynamic-graph update lowers d^(1-b)),
    // so update pushes keep the reference's touched-only rule (allow_dense = 0).
    const bool dense_next =
        global || (a.allow_dense && ts.union_vol[par] * (double)a.dense_div > (double)n);
    const bool track = !dense_next && !sh.final_level && !(method == M_HK_TAYLOR && hk_last_level(sh));
    const bool tgt_scale = (kind == KIND_IGN);
    const int stamp = sh.stamp;
    // the last Taylor level only adds r into x (hk_solver.py:74-75): no push
    const bool no_push = (method == M_HK_TAYLOR) && hk_last_level(sh);

    // ---- long rows: one CTA per chunk of a.chunk edges ----
    if (sh.large_cnt > 0 && !no_push) {
        for (int k = blockIdx.x; k < sh.large_cnt; k += gridDim.x) {
            int2 e = blarge[k];
            int u = front[e.x];
            int64_t rp = g.row_ptr[u];
            int len = g.row_len[u];
            int beg = e.y * a.chunk;
            int end = min(len, beg + a.chunk);
            Vec<T, VEC> p;
            vload<T, VEC>(Pw + (int64_t)e.x * W + c0, p);
            const int gidx = threadIdx.x / L;
            for (int j0 = beg; j0 < end; j0 += kThreads / L) {
                int j = j0 + gidx;
                bool ok = j < end;
                int v = ok ? g.col[rp + j] : 0;
                if (ok) push_edge<T, VEC>(g, Tgt, a.ld, c0, v, p, tgt_scale);
                if (track) append_once(ok && lane_g == 0, v, mark, stamp, next, next_cnt, kFull);
            }
        }
    }
    // ---- medium rows: one warp per row ----
    if (sh.med_cnt > 0 && !no_push) {
        const int64_t gw = (int64_t)blockIdx.x * kWarps + warp;
        const int64_t nw = (int64_t)gridDim.x * kWarps;
        const int64_t wstart = (gw + (int64_t)t * 131) % nw;
        for (int64_t k = wstart; k < sh.med_cnt; k += nw) {
            int f = bmed[k];
            int u = front[f];
            int64_t rp = g.row_ptr[u];
            int len = g.row_len[u];
            Vec<T, VEC> p;
            vload<T, VEC>(Pw + (int64_t)f * W + c0, p);
            for (int j0 = 0; j0 < len; j0 += GPW) {
                int j = j0 + grp_w;
                bool ok = j < len;
                int v = ok ? g.col[rp + j] : 0;
                if (ok) push_edge<T, VEC>(g, Tgt, a.ld, c0, v, p, tgt_scale);
                if (track) append_once(ok && lane_g == 0, v, mark, stamp, next, next_cnt, kFull);
            }
        }
    }
    // ---- short rows: one lane group per row ----
    if (sh.small_cnt > 0 && !no_push) {
        const int64_t nw = (int64_t)gridDim.x * kWarps;
        const int64_t wstart = (((int64_t)blockIdx.x * kWarps + warp) + (int64_t)t * 131) % nw;
        for (int64_t kb = wstart * GPW; kb < sh.small_cnt; kb += nw * GPW) {
            int64_t k = kb + grp_w;
            bool okr = k < sh.small_cnt;
            int len = 0;
            int64_t rp = 0;
            Vec<T, VEC> p;
#pragma unroll
            for (int i = 0; i < VEC; ++i) p.v[i] = T(0);
            if (okr) {
                int f = bsmall[k];
                int u = front[f];
                rp = g.row_ptr[u];
                len = g.row_len[u];
                vload<T, VEC>(Pw + (int64_t)f * W + c0, p);
            }
            int maxlen = len;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) maxlen = max(maxlen, __shfl_xor_sync(kFull, maxlen, o));
            for (int j = 0; j < maxlen; ++j) {
                bool ok = j < len;
                int v = ok ? g.col[rp + j] : 0;
                if (ok) push_edge<T, VEC>(g, Tgt, a.ld, c0, v, p, tgt_scale);
                if (track) append_once(ok && lane_g == 0, v, mark, stamp, next, next_cnt, kFull);
            }
        }
    }
    // ---- HK: drop this level's sub-threshold residuals (hk_solver.py:284) ----
    if (hk) {
        T* Rcur = slab_ptr<T>((sh.level & 1) ? a.R2 : a.R, a, t);
        if (sh.dense) {
            for (int64_t u = (int64_t)blockIdx.x * kThreads + threadIdx.x; u < n; u += (int64_t)gridDim.x * kThreads)
                for (int c = 0; c < W; ++c) Rcur[u * a.ld + c] = T(0);
        } else {
            const int32_t* cand = a.cand + ((int64_t)t * 2 + par) * n;
            for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < sh.cand_cnt;
                 i += (int64_t)gridDim.x * kThreads) {
                int u = cand[i];
                for (int c = 0; c < W; ++c) Rcur[(int64_t)u * a.ld + c] = T(0);
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ts.dense_next[par ^ 1] = dense_next ? 1 : 0;
        atomicAdd(&a.stats->rounds, 1ull);
        if (dense_next) atomicAdd(&a.stats->dense_rounds, 1ull);
    }
}

// Round bookkeeping by block 0 (fields read only at the next round start):
// a local column with no active node this round is finished
// (ppr_solver.py:266-267); a global column whose CHECK found nothing above
// threshold is finished (:292-293); HK stops after its last level
// (hk_solver.py:235); a tile is done when its frontier is empty.
template <int W>
__device__ void finish_round(const PushArgs& a, int t, const TileSh& sh) {
    if (blockIdx.x != 0) return;
    const int m = sh.tp.method;
    const bool gcheck = (m == M_GLOBAL_GD || m == M_GLOBAL_CHEBY);
    const bool hk_end = method_is_hk(m) && hk_last_level(sh);
    if (threadIdx.x < W && threadIdx.x < sh.tp.ncols) {
        ColState& cs = a.cs[(int64_t)t * W + threadIdx.x];
        if (cs.live) {
            bool worked = gcheck ? (cs.check_cnt[sh.parity] > 0) : (cs.round_active[sh.parity] > 0);
            if (method_is_hk(m) && m != M_HK_LOCAL) worked = true;  // fixed sweeps per level
            if (worked) cs.rounds += 1;
            if (!worked || hk_end) {
                cs.live = 0;
                cs.finish_ns = globaltimer_ns();
            }
        }
    }
    if (threadIdx.x == 0) {
        if (a.ts[t].front_cnt[sh.parity] == 0 || hk_end) a.ts[t].done = 1;
    }
}

template <typename T, int W>
__global__ void __launch_bounds__(kThreads) push_kernel(PushArgs a) {
    __shared__ TileSh sh;
    __shared__ PrepSh ps;
    __shared__ int s_cnt[kMaxW];
    __shared__ unsigned s_live[kMaxTiles / 32];
    __shared__ int s_any, s_check;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.stats->start_ns = globaltimer_ns();
    int it = 0;
    for (; it < a.round_budget; ++it) {
        // ---- snapshot of live tiles for this round ----
        if (threadIdx.x == 0) { s_any = 0; s_check = 0; }
        for (int w = threadIdx.x; w < (a.ntiles + 31) / 32; w += kThreads) s_live[w] = 0;
        __syncthreads();
        for (int t = threadIdx.x; t < a.ntiles; t += kThreads) {
            const TileState& ts = a.ts[t];
            bool live = !ts.done && (ts.round + it) < a.max_rounds;
            if (live) {
                atomicOr(&s_live[t >> 5], 1u << (t & 31));
                int m = a.tp[t].method;
                if (m == M_GLOBAL_GD || m == M_GLOBAL_CHEBY) s_check = 1;
                s_any = 1;
            }
        }
        __syncthreads();
        if (!s_any) break;
        const bool timer = (blockIdx.x == 0 && threadIdx.x == 0);
        unsigned long long t0 = timer ? globaltimer_ns() : 0ull;
        // ---- CHECK (global GD / Chebyshev tiles) ----
        if (s_check) {
            for (int t = 0; t < a.ntiles; ++t) {
                if (!(s_live[t >> 5] & (1u << (t & 31)))) continue;
                int m = a.tp[t].method;
                if (m != M_GLOBAL_GD && m != M_GLOBAL_CHEBY) continue;
                check_phase<T, W>(a, t, it, s_cnt);
            }
            if (!grid_barrier(a.bar, a.err)) return;
            if (timer) {
                unsigned long long t1 = globaltimer_ns();
                a.stats->check_ns += t1 - t0;
                t0 = t1;
            }
        }
        // ---- PREP ----
        for (int t = 0; t < a.ntiles; ++t) {
            if (!(s_live[t >> 5] & (1u << (t & 31)))) continue;
            load_tile<W>(a, t, it, sh);
            prep_phase<T, W>(a, t, sh, ps);
        }
        if (!grid_barrier(a.bar, a.err)) return;
        if (timer) {
            unsigned long long t1 = globaltimer_ns();
            a.stats->prep_ns += t1 - t0;
            t0 = t1;
        }
        // ---- SCATTER + bookkeeping ----
        for (int t = 0; t < a.ntiles; ++t) {
            if (!(s_live[t >> 5] & (1u << (t & 31)))) continue;
            load_tile<W>(a, t, it, sh);
            if (sh.front_cnt > 0) scatter_phase<T, W>(a, t, sh);
            finish_round<W>(a, t, sh);
            __syncthreads();
        }
        if (!grid_barrier(a.bar, a.err)) return;
        if (timer) a.stats->scatter_ns += globaltimer_ns() - t0;
    }
    // Record the rounds advanced by this launch (all blocks are past their
    // last read of ts.round once the final barrier completes).
    if (it > 0 && !grid_barrier(a.bar, a.err)) return;
    if (blockIdx.x == 0) {
        for (int t = threadIdx.x; t < a.ntiles; t += kThreads) {
            TileState& ts = a.ts[t];
            if (!ts.done) ts.round = min(ts.round + it, a.max_rounds);
        }
    }
}

}  // namespace

// Host-side launcher: picks the instantiation for (T, W) and launches it
// cooperatively with the largest co-resident grid.
template <typename T, int W>
static cudaError_t launch_t(const PushArgs& a, int grid, cudaStream_t st) {
    void* args[] = {const_cast<PushArgs*>(&a)};
    return cudaLaunchCooperativeKernel((void*)push_kernel<T, W>, dim3(grid), dim3(kThreads), args, 0, st);
}

template <typename T, int W>
static int max_grid_t(int sms) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, push_kernel<T, W>, kThreads, 0);
    return per_sm * sms;
}

int engine_max_grid(int prec64, int W, int sms) {
    if (prec64) {
        switch (W) {
            case 1: return max_grid_t<double, 1>(sms);
            case 2: return max_grid_t<double, 2>(sms);
            case 4: return max_grid_t<double, 4>(sms);
            case 8: return max_grid_t<double, 8>(sms);
            case 16: return max_grid_t<double, 16>(sms);
            case 32: return max_grid_t<double, 32>(sms);
        }
    } else {
        switch (W) {
            case 1: return max_grid_t<float, 1>(sms);
            case 2: return max_grid_t<float, 2>(sms);
            case 4: return max_grid_t<float, 4>(sms);
            case 8: return max_grid_t<float, 8>(sms);
            case 16: return max_grid_t<float, 16>(sms);
            case 32: return max_grid_t<float, 32>(sms);
        }
    }
    return 0;
}

cudaError_t engine_launch(const PushArgs& a, int prec64, int W, int grid, cudaStream_t st) {
    if (prec64) {
        switch (W) {
            case 1: return launch_t<double, 1>(a, grid, st);
            case 2: return launch_t<double, 2>(a, grid, st);
            case 4: return launch_t<double, 4>(a, grid, st);
            case 8: return launch_t<double, 8>(a, grid, st);
            case 16: return launch_t<double, 16>(a, grid, st);
            case 32: return launch_t<double, 32>(a, grid, st);
        }
    } else {
        switch (W) {
            case 1: return launch_t<float, 1>(a, grid, st);
            case 2: return launch_t<float, 2>(a, grid, st);
            case 4: return launch_t<float, 4>(a, grid, st);
            case 8: return launch_t<float, 8>(a, grid, st);
            case 16: return launch_t<float, 16>(a, grid, st);
            case 32: return launch_t<float, 32>(a, grid, st);
        }
    }
    return cudaErrorInvalidValue;
}

}  // namespace gde
