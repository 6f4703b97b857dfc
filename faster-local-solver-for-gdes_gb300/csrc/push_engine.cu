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

// Resident blocks per SM requested from the compiler (bounds registers) and
// independent edges in flight per lane in the W = 1 scatter; both can be
// overridden at build time for tuning.  FP32 kernels of up to 8 columns
// trade a few spilled bytes for a fourth block per SM: their memory-latency-
// bound phases gain more from the extra warps (served PPR +3 to +7%, the
// 8-column InstantGNN push +4%) than the spills cost; 16- and 32-column and
// FP64 kernels spill more and keep three.  The one-column FP32 kernel (the
// served slots) runs five blocks per SM with two edges in flight per lane:
// with a barrier per slot group, more resident warps each with fewer
// outstanding atomics beat fewer warps with more (2,647 -> 2,740-2,800
// queries/s on the 2.36M-node workload; four edges per lane at five or six
// blocks, or one or two at seven blocks with their spills, measured slower).
#ifndef GDE_MIN_BLOCKS
#define GDE_MIN_BLOCKS 3
#endif
#ifndef GDE_MIN_BLOCKS_F32
#define GDE_MIN_BLOCKS_F32 4
#endif
#ifndef GDE_MIN_BLOCKS_W1
#define GDE_MIN_BLOCKS_W1 5
#endif
#ifndef GDE_VEC_COLS
#define GDE_VEC_COLS 0  // 1: 128-bit column-word loads for rows of 128 edges and more (W = 1)
#endif
#ifndef GDE_EDGE_ILP
#define GDE_EDGE_ILP 2
#endif

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// Threshold test r >= theta * d without FP64 arithmetic in the common case.
// GB300 issues FP64 at a small fraction of the FP32 rate, so the FP32 path
// decides in FP32 whenever r is clearly on one side: t32 = fl32(fl32(theta) *
// d) is within 2^-23 (relative) of theta * d for an integer degree d < 2^24,
// so r >= t32 * (1 + 2^-20) implies r > theta * d and r < t32 * (1 - 2^-20)
// implies r < theta * d.  Only inside that band is the FP64 product formed.
// The result is exactly that of (double)r >= theta * d.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool ge_threshold(float r, float t32, double theta, double d) {
    if (r >= t32 * (1.f + 0x1p-20f)) return true;
    if (r < t32 * (1.f - 0x1p-20f)) return false;
    return (double)r >= theta * d;
}

// The same decision for a threshold that is not theta times an integer
// degree (InstantGNN's theta d^(1-beta), the heat kernel's theta d / (N psi)):
// t32 is its FP32 approximation, within 2^-21 (relative) of the FP64 value
// thr64() -- a few roundings of 2^-24 each -- so the 2^-20 band still
// brackets it, and thr64() is evaluated only inside the band.
template <typename F>
__device__ __forceinline__ bool ge_band(float r, float t32, F thr64) {
    if (r >= t32 * (1.f + 0x1p-20f)) return true;
    if (r < t32 * (1.f - 0x1p-20f)) return false;
    return (double)r >= thr64();
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

// atomic add of VEC contiguous values returning the previous values
template <typename T, int VEC>
__device__ __forceinline__ void vatomic_ret(T* p, const Vec<T, VEC>& o, Vec<T, VEC>& old) {
#pragma unroll
    for (int i = 0; i < VEC; ++i) old.v[i] = (o.v[i] != T(0)) ? atomicAdd(p + i, o.v[i]) : T(0);
}
template <>
__device__ __forceinline__ void vatomic_ret<float, 4>(float* p, const Vec<float, 4>& o, Vec<float, 4>& old) {
    float4 r = atomicAdd(reinterpret_cast<float4*>(p), make_float4(o.v[0], o.v[1], o.v[2], o.v[3]));
    old.v[0] = r.x; old.v[1] = r.y; old.v[2] = r.z; old.v[3] = r.w;
}
template <>
__device__ __forceinline__ void vatomic_ret<float, 2>(float* p, const Vec<float, 2>& o, Vec<float, 2>& old) {
    float2 r = atomicAdd(reinterpret_cast<float2*>(p), make_float2(o.v[0], o.v[1]));
    old.v[0] = r.x; old.v[1] = r.y;
}

template <typename T>
__device__ __forceinline__ T* slab_ptr(void* base, const PushArgs& a, int t) {
    return reinterpret_cast<T*>(base) + (int64_t)t * a.tile_stride;
}

// The solution and its Kahan term may be interleaved ({x, c} per node, one
// sector per random access): their own row stride and tile offset.
__device__ __forceinline__ int64_t x_ld(const PushArgs& a) { return a.xld ? a.xld : a.ld; }
template <typename T>
__device__ __forceinline__ T* xslab_ptr(void* base, const PushArgs& a, int t) {
    const int64_t s = a.xq ? a.ts[t].qid : t;  // served with per-query solution slabs
    return reinterpret_cast<T*>(base) + s * (a.xld ? a.xtile : a.tile_stride);
}

// FP64 residual of the hub prefix of slot t (served FP32 crossing slots), or nullptr.
__device__ __forceinline__ double* rh_ptr(const PushArgs& a, int t) {
    return a.RH ? a.RH + (int64_t)t * a.rh_cut : nullptr;
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
    int col_sweeps[kMaxW];  // HK global sweeps with omega != 1: sweeps of this level
};

// HK relaxation (hk_solver.py:248-264, :266-280): a push moves omega r into
// the solution and the next level and keeps r - omega r at this level.  The
// node pushes `fixed` times (global sweeps), or while its residual stays at
// or above thr (local queue); returns the total moved, the sub-pushes and
// the residual left, which the level then drops (:284).
__device__ __forceinline__ double hk_relax(double r, double omega, double thr, int fixed, int* subs, double* left) {
    double moved = 0.0;
    int s = 0;
    do {
        const double ru = omega * r;
        moved += ru;
        r -= ru;
        ++s;
    } while (s < kMaxRelax && (fixed > 0 ? s < fixed : fabs(r) >= thr));
    *subs = s;
    *left = r;
    return moved;
}

__device__ __forceinline__ bool is_absorbing(const DevGraph& g, int u) {
    int len = g.row_len[u];
    return len == 0 || (len == 1 && g.col[g.row_ptr[u]] == u);
}

// Load the state of tile t at launch iteration `it` (block-wide).
template <int W>
__device__ void load_tile(const PushArgs& a, int t, int it, TileSh& sh) {
    if (threadIdx.x == 0) {
        const TileState& ts = a.ts[t];
        sh.tp = a.tp[t];
        sh.level = it - ts.t0;
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
        sh.col_sweeps[threadIdx.x] = max(1, c.hk_sweeps[sh.parity]);
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// HK global sweeps with omega != 1 (hk_solver.py:266-280): a level repeats
// its sweep over all nodes until no residual is at or above threshold, so
// every node takes the same number of sweeps, the most any node needs.  This
// phase finds that number before the level's PREP pushes.
// ---------------------------------------------------------------------------
template <typename T, int W>
__device__ void hk_sweeps_phase(const PushArgs& a, int t, int it) {
    constexpr int VEC = (sizeof(T) == 4) ? (W >= 4 ? 4 : W) : (W >= 2 ? 2 : 1);
    constexpr int L = W / VEC;
    __shared__ int s_live[kMaxW];
    __shared__ double s_theta[kMaxW];
    __shared__ int s_max[kMaxW];
    const int64_t n = a.g.n;
    const TileParams& tp = a.tp[t];
    const int level = it - a.ts[t].t0;
    const int par = level & 1;
    const T* R = slab_ptr<T>(par ? a.R2 : a.R, a, t);
    const double psi = tp.psi_tab[level];
    const double nl = (double)tp.n_levels;
    if (threadIdx.x < W) {
        const ColState& c = a.cs[(int64_t)t * W + threadIdx.x];
        s_live[threadIdx.x] = (threadIdx.x < tp.ncols) && c.live;
        s_theta[threadIdx.x] = c.theta;
        s_max[threadIdx.x] = 1;
    }
    __syncthreads();
    const int c0 = (threadIdx.x % L) * VEC;
    int mx[VEC];
#pragma unroll
    for (int i = 0; i < VEC; ++i) mx[i] = 1;
    const int64_t gid = ((int64_t)blockIdx.x * kThreads + threadIdx.x) / L;
    const int64_t ng = (int64_t)gridDim.x * kThreads / L;
    for (int64_t u = gid; u < n; u += ng) {
        Vec<T, VEC> rv;
        vload<T, VEC>(R + u * a.ld + c0, rv);
        const double d = a.g.degd[u];
#pragma unroll
        for (int i = 0; i < VEC; ++i) {
            const double r = (double)rv.v[i];
            if (!s_live[c0 + i] || r == 0.0) continue;
            const double thr = ((s_theta[c0 + i] * d) / nl) / psi;
            int subs;
            double left;
            hk_relax(r, tp.omega, thr, 0, &subs, &left);
            mx[i] = max(mx[i], subs);
        }
    }
#pragma unroll
    for (int i = 0; i < VEC; ++i)
        if (mx[i] > 1) atomicMax(&s_max[c0 + i], mx[i]);
    __syncthreads();
    if (threadIdx.x < W && s_max[threadIdx.x] > 1)
        atomicMax(&a.cs[(int64_t)t * W + threadIdx.x].hk_sweeps[par], s_max[threadIdx.x]);
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
    __shared__ float s_theta_f[kMaxW];
    __shared__ int s_par;
    const int64_t n = a.g.n;
    const T* R = slab_ptr<T>(a.R, a, t);
    if (threadIdx.x == 0) s_par = (it - a.ts[t].t0) & 1;
    if (threadIdx.x < W) {
        const ColState& c = a.cs[(int64_t)t * W + threadIdx.x];
        s_live[threadIdx.x] = (threadIdx.x < a.tp[t].ncols) && c.live;
        s_theta[threadIdx.x] = c.theta;
        s_theta_f[threadIdx.x] = (float)c.theta;
        s_cnt[threadIdx.x] = 0;
    }
    __syncthreads();
    // FP32 tiles on integer degrees test in FP32 (exact through the band of
    // ge_threshold) and read the 4-byte degree: FP64 is a small fraction of
    // the FP32 rate on GB300, and this phase touches every node.
    const bool f32 = (sizeof(T) == 4) && a.g.degf_exact;
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
        if (f32) {
            const float df = a.g.degf[u];
#pragma unroll
            for (int i = 0; i < VEC; ++i)
                cnt[i] += (s_live[c0 + i] && ge_threshold(fabsf((float)rv.v[i]), s_theta_f[c0 + i] * df,
                                                          s_theta[c0 + i], (double)df)) ? 1 : 0;
        } else {
            double d = a.g.degd[u];
#pragma unroll
            for (int i = 0; i < VEC; ++i) {
                double thr = s_theta[c0 + i] * d;
                cnt[i] += (s_live[c0 + i] && fabs((double)rv.v[i]) >= thr) ? 1 : 0;
            }
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
// Work distribution.  Each phase flattens its work over all live tiles
// (candidates for PREP; short rows, medium rows and long-row chunks for
// SCATTER) and gives every block one contiguous, equal share of each
// flattened space, so a round's work is balanced over the whole GPU no
// matter how it is spread over tiles, and a block touches only the one or
// two tiles its share overlaps.
// ---------------------------------------------------------------------------
constexpr int kMaxLaunchTiles = 512;

struct RoundSh {
    int ntl;                                    // live tiles this round
    int any_check;                              // some live tile needs a CHECK phase
    int any_idle;                               // served solves: some slot awaits a query
    int tiles[kMaxLaunchTiles];                 // live tile ids (ascending)
    unsigned char idle[kMaxLaunchTiles];        // 1: slot idle at the round start; 2: draining (online)
    short drain[kMaxLaunchTiles];               // online slots to clear this round (SLOT_DRAIN)
    int ndrain;
    long long off[4][kMaxLaunchTiles + 1];      // exclusive prefix sums of the current phase's spaces
    int level[kMaxLaunchTiles];                 // per live tile: rounds since its start
    unsigned char flags[kMaxLaunchTiles];       // per live tile scatter flags (SF_*)
    long long scan_tmp[kWarps];
};

enum : unsigned char { SF_FINAL = 1, SF_TRACK = 2, SF_NOPUSH = 4, SF_TGTSCALE = 8, SF_HK = 16, SF_CROSS = 32 };

// Local GD for PPR and Katz only ever adds non-negative values to
// non-negative residuals, so a node enters the next frontier exactly when one
// of the round's additions takes it from below its threshold to at or above
// it -- the reference's own enqueue test right after `rt[v] += val`
// (ppr_solver.py:284-288).  Such tiles append on the crossing, never scan
// densely, and PREP visits exactly the frontier.
__device__ __forceinline__ bool tile_crosses(const TileParams& tp) {
    return tp.method == M_LOCAL_GD && (tp.kind == KIND_PPR || tp.kind == KIND_KATZ);
}

// Does tile t's next round scan every node?  (identical in every block)
__device__ __forceinline__ bool dense_next_round(const PushArgs& a, const TileParams& tp, const TileState& ts,
                                                 int par) {
    if (method_is_global(tp.method)) return true;
    if (tile_crosses(tp) || !a.allow_dense) return false;
    return ts.union_vol[par] * (double)a.dense_div > (double)a.g.n;
}

// Exclusive prefix over vals[0..m) (m <= 512) written to out[0..m]; block-wide.
__device__ void block_exclusive_scan(const long long* vals, int m, long long* out, long long* tmp) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    long long v0 = (2 * tid < m) ? vals[2 * tid] : 0;
    long long v1 = (2 * tid + 1 < m) ? vals[2 * tid + 1] : 0;
    long long s = v0 + v1;
    long long inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(kFull, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) tmp[warp] = inc;
    __syncthreads();
    if (tid == 0) {
        long long acc = 0;
        for (int w = 0; w < kWarps; ++w) {
            long long c = tmp[w];
            tmp[w] = acc;
            acc += c;
        }
        out[m] = acc;
    }
    __syncthreads();
    long long excl = tmp[warp] + inc - s;
    if (2 * tid < m) out[2 * tid] = excl;
    if (2 * tid + 1 < m) out[2 * tid + 1] = excl + v0;
    __syncthreads();
}

// First live-tile index k with off[k+1] > x (off ascending, off[0] = 0).
__device__ __forceinline__ int find_tile(const long long* off, int ntl, long long x) {
    int lo = 0, hi = ntl - 1;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (off[mid + 1] > x) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}


// The block group this block belongs to (served launches with a.groups > 1
// split the grid; every other launch is one group): group g holds blocks
// [ceil(g B / G), ceil((g+1) B / G)).
struct GroupInfo {
    int id;   // group index
    int blk;  // this block's index within the group
    int dim;  // blocks in the group
};
__device__ __forceinline__ GroupInfo group_of(const PushArgs& a) {
    const int G = a.groups > 1 ? a.groups : 1;
    const long long B = (long long)gridDim.x - (a.serve ? a.queue.sp_blocks : 0);  // the dense blocks
    const int g = (int)((long long)blockIdx.x * G / B);
    const int start = (int)(((long long)g * B + G - 1) / G);
    const int end = (int)(((long long)(g + 1) * B + G - 1) / G);
    return GroupInfo{g, (int)blockIdx.x - start, end - start};
}

// This block's share [lo, hi) of a flattened space of `total` items (its group's blocks split it).
__device__ __forceinline__ void block_share(long long total, long long& lo, long long& hi, const GroupInfo& gi) {
    lo = total * (long long)gi.blk / gi.dim;
    hi = total * (long long)(gi.blk + 1) / gi.dim;
}

// ---------------------------------------------------------------------------
// PREP over candidates [beg, end) of tile t.
// ---------------------------------------------------------------------------
struct PrepSh {
    double col_oper[kMaxW];
    int col_nodes[kMaxW];
    double vol;
    int nodes;
    // this block's launch totals (LaunchStats fields), flushed at kernel end
    unsigned long long acc_col_nodes, acc_union_nodes;
    double acc_col_vol, acc_union_vol;
};

// Frontier compaction of one node per lane (W = 1): front index, degree
// bucket, work items and the push row P[fidx].
template <typename T>
__device__ __forceinline__ void emit_node_w1(const PushArgs& a, int t, int par, bool node_in, int len, long long rp,
                                             T push) {
    const int lane = threadIdx.x & 31;
    const int64_t n = a.g.n;
    TileState& ts = a.ts[t];
    const unsigned bf = __ballot_sync(kFull, node_in);
    if (bf == 0) return;
    int bucket = -1, nch = 0;
    if (node_in) {
        if (len <= a.small_max) bucket = 0;
        else if (len <= a.med_max) bucket = 1;
        else { bucket = 2; nch = (len + a.chunk - 1) / a.chunk; }
    }
    const unsigned bs = __ballot_sync(kFull, bucket == 0);
    const unsigned bm = __ballot_sync(kFull, bucket == 1);
    int sc = nch;  // inclusive warp scan of chunk counts
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, sc, o);
        if (lane >= o) sc += y;
    }
    const int wch = __shfl_sync(kFull, sc, 31);
    int b0 = 0, b1 = 0, b2 = 0, b3 = 0;
    if (lane == 0) {
        b0 = atomicAdd(&ts.front_cnt[par], __popc(bf));
        if (bs) b1 = atomicAdd(&ts.small_cnt[par], __popc(bs));
        if (bm) b2 = atomicAdd(&ts.med_cnt[par], __popc(bm));
        if (wch) b3 = atomicAdd(&ts.large_cnt[par], wch);
    }
    b0 = __shfl_sync(kFull, b0, 0);
    b1 = __shfl_sync(kFull, b1, 0);
    b2 = __shfl_sync(kFull, b2, 0);
    b3 = __shfl_sync(kFull, b3, 0);
    if (!node_in) return;
    const unsigned below = (1u << lane) - 1u;
    const int fidx = b0 + __popc(bf & below);
    PushItem item;
    item.rp = rp;
    item.len = len;
    item.fidx = fidx;
    PushItem* bsmall = a.bsmall + (int64_t)t * n;
    if (bucket == 0) {
        bsmall[b1 + __popc(bs & below)] = item;
    } else if (bucket == 1) {
        bsmall[(n - 1) - (b2 + __popc(bm & below))] = item;
    } else {
        PushItem* blarge = a.blarge + (int64_t)t * a.large_cap;
        const int lb = b3 + (sc - nch);
        for (int ch = 0; ch < nch; ++ch) {
            item.rp = rp + (long long)ch * a.chunk;
            item.len = min(a.chunk, len - ch * a.chunk);
            blarge[lb + ch] = item;
        }
    }
    reinterpret_cast<T*>(a.P)[(int64_t)t * n + fidx] = push;
}

// PREP of a W = 1 PPR/Katz local GD tile over candidates [beg, end): the
// candidates are exactly last round's threshold crossings.  Each lane takes
// kPrepILP candidates and issues every per-node load (residual, degree,
// solution, Kahan term, row start and length) before using any of them.
#ifndef GDE_PREP_ILP
#define GDE_PREP_ILP 2
#endif
constexpr int kPrepILP = GDE_PREP_ILP;

template <typename T>
__device__ void prep_w1_cross(const PushArgs& a, int t, const TileSh& sh, long long beg, long long end,
                              double& my_oper, int& my_nodes, double& my_vol, int& my_cnt) {
    const DevGraph& g = a.g;
    const int64_t n = g.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int par = sh.parity;
    const int32_t* cand = a.cand + ((int64_t)t * 2 + par) * n;
    T* R = slab_ptr<T>(a.R, a, t);
    T* X = xslab_ptr<T>(a.X, a, t);
    float* XC = a.kahan ? xslab_ptr<float>(a.XC, a, t) : nullptr;
    const int64_t xld = x_ld(a);
    const double alpha = sh.tp.alpha;
    const bool katz = sh.tp.kind == KIND_KATZ;
    const double theta = sh.col_theta[0];
    const float theta_f = (float)theta;
    const float alpha_f = (float)alpha, omalpha_f = (float)(1. - alpha);
    const int64_t ld = a.ld;
    double* RH = (sizeof(T) == 4) ? rh_ptr(a, t) : nullptr;  // hub prefix in FP64
    const int rh_cut = a.rh_cut;
    long long ideg = 0;  // sum of (integer) degrees of the pushed nodes
    for (long long base = beg + (long long)warp * 32 * kPrepILP; base < end;
         base += (long long)kWarps * 32 * kPrepILP) {
        bool val[kPrepILP];
        int u[kPrepILP];
#pragma unroll
        for (int q = 0; q < kPrepILP; ++q) {
            const long long i = base + q * 32 + lane;
            val[q] = i < end;
            u[q] = val[q] ? cand[i] : 0;
        }
        T r[kPrepILP], xv[kPrepILP];
        double rd[kPrepILP];  // the FP64 residual of a hub-prefix node (RH), else unused
        float df[kPrepILP], xc[kPrepILP];
        int len[kPrepILP];
        long long rp[kPrepILP];
#pragma unroll
        for (int q = 0; q < kPrepILP; ++q) {
            r[q] = T(0); rd[q] = 0.0; xv[q] = T(0); df[q] = 1.f; xc[q] = 0.f; len[q] = 0; rp[q] = 0;
            if (val[q]) {
                const int64_t off = (int64_t)u[q] * ld, xoff = (int64_t)u[q] * xld;
                if (RH && u[q] < rh_cut) {
                    rd[q] = RH[u[q]];
                    r[q] = (T)rd[q];
                } else {
                    r[q] = R[off];
                }
                xv[q] = X[xoff];
                if (XC) xc[q] = XC[xoff];
                if (g.rec) {
                    const NodeRec nr = g.rec[u[q]];
                    rp[q] = nr.rp;
                    len[q] = nr.len;
                    df[q] = nr.degf;
                } else {
                    df[q] = g.degf[u[q]];
                    len[q] = g.row_len[u[q]];
                    rp[q] = g.row_ptr[u[q]];
                }
            }
        }
#pragma unroll
        for (int q = 0; q < kPrepILP; ++q) {
            bool act = false;
            T push = T(0);
            if (val[q]) {
                const double du = g.degf_exact ? (double)df[q] : g.degd[u[q]];
                if constexpr (sizeof(T) == 4) {
                    if (RH && u[q] < rh_cut) {
                        // hub prefix: FP64 residual, FP64 test and push value
                        act = fabs(rd[q]) >= theta * du;
                        if (act) push = (T)(katz ? alpha * rd[q] : ((1. - alpha) * rd[q]) / du);
                    } else {
                        // FP32 tile: exact threshold test mostly in FP32; push value in FP32
                        if (g.degf_exact) act = ge_threshold(fabsf(r[q]), theta_f * df[q], theta, du);
                        else act = fabs((double)r[q]) >= theta * du;
                        if (act) push = katz ? alpha_f * r[q] : (omalpha_f * r[q]) / df[q];
                    }
                } else {
                    const double rv = (double)r[q];
                    act = fabs(rv) >= theta * du;
                    // ppr_solver.py:276-281 / katz_solver.py:226-231
                    if (act) push = (T)(katz ? alpha * rv : ((1. - alpha) * rv) / du);
                }
                if (act) {
                    const int64_t off = (int64_t)u[q] * ld, xoff = (int64_t)u[q] * xld;
                    if (RH && u[q] < rh_cut) RH[u[q]] = 0.0;
                    else R[off] = T(0);
                    if (XC) {
                        // Kahan-compensated FP32 accumulation of the solution
                        const float y = (float)r[q] - xc[q];
                        const float s = (float)xv[q] + y;
                        XC[xoff] = (s - (float)xv[q]) - y;
                        X[xoff] = (T)s;
                    } else {
                        X[xoff] = xv[q] + r[q];
                    }
                    my_nodes += 1;
                    if (g.degf_exact) ideg += (long long)df[q];
                    else { my_oper += du; my_vol += du; }
                    my_cnt += 1;
                }
            }
            emit_node_w1<T>(a, t, par, act, len[q], rp[q], push);
        }
    }
    my_oper += (double)ideg;
    my_vol += (double)ideg;
}

template <typename T, int W>
__device__ void prep_range(const PushArgs& a, int t, const TileSh& sh, PrepSh& ps, long long beg, long long end) {
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
    const int lane_g = lane % L, grp_w = lane / L;
    const int c0 = lane_g * VEC;
    const int32_t* cand = a.cand + ((int64_t)t * 2 + par) * n;
    int32_t* next = a.cand + ((int64_t)t * 2 + (par ^ 1)) * n;
    int32_t* mark = a.mark + (int64_t)t * n;
    T* Pw = reinterpret_cast<T*>(a.P) + (int64_t)t * n * W;
    PushItem* bsmall = a.bsmall + (int64_t)t * n;       // short rows grow up from 0,
    PushItem* bmed_end = bsmall + (n - 1);               // medium rows down from n-1
    PushItem* blarge = a.blarge + (int64_t)t * a.large_cap;
    TileState& ts = a.ts[t];
    T* R = slab_ptr<T>((hk && (sh.level & 1)) ? a.R2 : a.R, a, t);
    T* X = xslab_ptr<T>(a.X, a, t);
    float* XC = a.kahan ? xslab_ptr<float>(a.XC, a, t) : nullptr;
    const int64_t xld = x_ld(a);
    T* DX = cheby ? slab_ptr<T>(a.DX, a, t) : nullptr;
    const double alpha = sh.tp.alpha;
    int* next_cnt = &ts.cand_cnt[(sh.level + 1) % 3];

    if (threadIdx.x < W) { ps.col_oper[threadIdx.x] = 0.0; ps.col_nodes[threadIdx.x] = 0; }
    if (threadIdx.x == 0) { ps.vol = 0.0; ps.nodes = 0; }
    __syncthreads();

    double my_oper[VEC];
    int my_nodes[VEC];
    double thr_scale[VEC];
    bool live[VEC];
    // FP32 tiles on integer degrees decide and push in FP32, as the W = 1
    // path does: each threshold test is exact through the FP64 band
    // (ge_band), and the push value is formed in FP32, the tile's precision.
    // FP64 is a small fraction of the FP32 rate on GB300, and a dense round
    // visits every node and column.  Chebyshev keeps its recurrence in FP64.
    const bool f32 = (sizeof(T) == 4) && g.degf_exact && !cheby;
    float thr_f[VEC];
    const double hk_div = hk ? (double)sh.tp.n_levels * sh.psi : 1.0;
#pragma unroll
    for (int k = 0; k < VEC; ++k) {
        my_oper[k] = 0.0;
        my_nodes[k] = 0;
        live[k] = sh.col_live[c0 + k] != 0;
        thr_scale[k] = sh.col_theta[c0 + k];
        thr_f[k] = (float)(hk ? thr_scale[k] / hk_div : thr_scale[k]);
    }
    const float alpha_f = (float)alpha, omalpha_f = (float)(1. - alpha), xgain_f = (float)sh.tp.x_gain;
    const float hkc_f = hk ? (float)(sh.tp.tau / ((double)sh.level + 1.)) : 0.f;
    double my_vol = 0.0;
    int my_cnt = 0;

    // A W = 1 crossing tile visits exactly the nodes that crossed their
    // threshold last round: every candidate is active, so all its loads are
    // issued at once (prep_w1_cross).
    bool fast = false;
    if constexpr (W == 1) fast = tile_crosses(sh.tp) && !sh.dense && live[0];
    if (fast) {
        if constexpr (W == 1) prep_w1_cross<T>(a, t, sh, beg, end, my_oper[0], my_nodes[0], my_vol, my_cnt);
    } else {
        for (long long base = beg + (long long)warp * GPW; base < end; base += (long long)kWarps * GPW) {
            const long long i = base + grp_w;
            const bool valid = i < end;
            int u = 0;
            bool act[VEC];
            Vec<T, VEC> push;
    #pragma unroll
            for (int k = 0; k < VEC; ++k) { act[k] = false; push.v[k] = T(0); }
            double du = 1.0;
            bool absorb = false;
            bool any = false;
            Vec<T, VEC> r;
            float df = 1.f;
            if (valid) {
                u = sh.dense ? (int)i : cand[i];
                const int64_t off = (int64_t)u * a.ld + c0;
                const int64_t xoff = (int64_t)u * xld + c0;
                vload<T, VEC>(R + off, r);
                // fast test first: most scanned nodes are below every threshold
                df = g.degf[u];
                du = g.degf_exact ? (double)df : g.degd[u];
                const double thr_base = (kind == KIND_IGN) ? g.nfac[u] : du;
                const float base_f = (kind == KIND_IGN) ? (float)thr_base : df;
    #pragma unroll
                for (int k = 0; k < VEC; ++k) {
                    if (!live[k]) continue;
                    bool a_k;
                    if (global) {
                        a_k = (r.v[k] != T(0));
                    } else if (f32) {
                        a_k = ge_band(fabsf((float)r.v[k]), thr_f[k] * base_f, [&] {
                            return hk ? ((thr_scale[k] * thr_base) / (double)sh.tp.n_levels) / sh.psi
                                      : thr_scale[k] * thr_base;
                        });
                    } else {
                        const double rv = (double)r.v[k];
                        double thr;
                        if (hk) thr = ((thr_scale[k] * thr_base) / (double)sh.tp.n_levels) / sh.psi;
                        else thr = thr_scale[k] * thr_base;
                        a_k = fabs(rv) >= thr;
                    }
                    act[k] = a_k;
                    any |= a_k;
                }
                if (cheby && global) {
                    // global Chebyshev updates every node whose three-term step is non-zero
                    Vec<T, VEC> dxv;
                    vload<T, VEC>(DX + off, dxv);
    #pragma unroll
                    for (int k = 0; k < VEC; ++k) {
                        if (!live[k]) continue;
                        act[k] = ((double)r.v[k] != 0.0) || ((double)dxv.v[k] != 0.0);
                        any |= act[k];
                    }
                }
                if (any) {
                    absorb = ign && is_absorbing(g, u);
                    const float npush_f = (f32 && kind == KIND_IGN) ? (float)g.npush[u] : 1.f;
                    Vec<T, VEC> dxv;
                    if (cheby) vload<T, VEC>(DX + off, dxv);
                    Vec<T, VEC> xadd;
                    bool wrote = false;
    #pragma unroll
                    for (int k = 0; k < VEC; ++k) {
                        xadd.v[k] = T(0);
                        if (!act[k]) continue;
                        const double rv = (double)r.v[k];
                        if (cheby) {
                            // ppr_solver.py:642-646 / katz_solver.py:407-411
                            double tmp;
                            if (kind == KIND_KATZ) tmp = sh.coef1 * rv - sh.coef2 * (double)dxv.v[k];
                            else tmp = sh.coef1 * rv + (sh.coef1 - 1.) * (double)dxv.v[k];
                            if (global && tmp == 0.0) { act[k] = false; continue; }
                            T tmpT = (T)tmp;
                            xadd.v[k] = tmpT;
                            dxv.v[k] = tmpT;
                            r.v[k] = (T)(rv - (double)tmpT);  // rt[u] += -delta_xt[u] (:657)
                            double pv = (kind == KIND_KATZ) ? alpha * (double)tmpT : ((1. - alpha) * (double)tmpT) / du;
                            push.v[k] = (T)pv;
                        } else {
                            // An absorbing node (threshold 0) is visited once by the
                            // reference's initial scan and never re-enqueued; with a
                            // zero residual it has nothing to absorb.
                            if (absorb && r.v[k] == T(0)) { act[k] = false; continue; }
                            if (f32) {
                                const float rf = (float)r.v[k];
                                float pvf;
                                if (kind == KIND_PPR || kind == KIND_UPPR) pvf = (omalpha_f * rf) / df;
                                else if (kind == KIND_KATZ) pvf = alpha_f * rf;
                                else if (kind == KIND_HK) pvf = sh.final_level ? rf / df : (hkc_f * rf) / df;
                                else pvf = (omalpha_f * rf) / npush_f;
                                push.v[k] = absorb ? T(0) : (T)pvf;
                                xadd.v[k] = (kind == KIND_IGN && !absorb) ? (T)(xgain_f * rf) : r.v[k];
                                r.v[k] = T(0);
                                wrote = true;
                                my_nodes[k] += 1;
                                if (!absorb) my_oper[k] += du;
                                continue;
                            }
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
                            if constexpr (sizeof(T) == 8) {  // HK relaxation runs in FP64 only (host-checked)
                                if (kind == KIND_HK && hk_relaxed(sh.tp)) {
                                    const double thr = ((thr_scale[k] * du) / (double)sh.tp.n_levels) / sh.psi;
                                    int subs;
                                    double left;
                                    const double moved = hk_relax(rv, sh.tp.omega, thr,
                                                                  global ? sh.col_sweeps[c0 + k] : 0, &subs, &left);
                                    if (sh.final_level) push.v[k] = moved / du;
                                    else push.v[k] = ((sh.tp.tau / ((double)sh.level + 1.)) * moved) / du;
                                    xadd.v[k] = moved;
                                    r.v[k] = left;
                                    my_oper[k] += (double)(subs - 1) * du;  // the first sub-push is counted below
                                }
                            }
                        }
                        wrote = true;
                        my_nodes[k] += 1;
                        if (!absorb) my_oper[k] += du;
                    }
                    if (wrote) {
                        vstore<T, VEC>(R + off, r);
                        if (cheby) vstore<T, VEC>(DX + off, dxv);
                        Vec<T, VEC> xv;
                        vload<T, VEC>(X + xoff, xv);
                        if (absorb) {
                            // p[u] = r[u]; r[u] = 0 for an absorbing node (InstantGNN.py:22-25)
    #pragma unroll
                            for (int k = 0; k < VEC; ++k)
                                if (act[k]) {
                                    xv.v[k] = xadd.v[k];
                                    if (XC) XC[xoff + k] = 0.f;
                                }
                        } else if (XC) {
                            // Kahan-compensated FP32 accumulation of the solution
                            Vec<float, VEC> cc;
                            vload<float, VEC>(XC + xoff, cc);
    #pragma unroll
                            for (int k = 0; k < VEC; ++k)
                                if (act[k]) {
                                    float y = (float)xadd.v[k] - cc.v[k];
                                    float s = (float)xv.v[k] + y;
                                    cc.v[k] = (s - (float)xv.v[k]) - y;
                                    xv.v[k] = (T)s;
                                }
                            vstore<float, VEC>(XC + xoff, cc);
                        } else {
    #pragma unroll
                            for (int k = 0; k < VEC; ++k)
                                if (act[k]) xv.v[k] = xv.v[k] + xadd.v[k];
                        }
                        vstore<T, VEC>(X + xoff, xv);
                    }
                    any = false;
    #pragma unroll
                    for (int k = 0; k < VEC; ++k) any |= act[k];
                }
            }
            // ---- node-level frontier decision (OR over the lane group) ----
            const unsigned bal = __ballot_sync(kFull, any);
            if (bal == 0) continue;  // warp-uniform: nothing active in this warp
            const unsigned gmask = ((L == 32) ? kFull : ((1u << L) - 1u)) << (grp_w * L);
            const bool node_act = valid && (bal & gmask) != 0;
            const bool leader = (lane_g == 0);
            // Chebyshev moves r[u] by -dx[u]: u itself is a candidate next round
            if (cheby && !global) append_once(leader && node_act, u, mark, sh.stamp, next, next_cnt, kFull);
            const bool node_in = node_act && !absorb;  // absorbed nodes do not push
            int len = 0;
            int nch = 0;
            long long rp = 0;
            int bucket = -1;  // 0 short, 1 medium, 2 long
            if (node_in && leader) {
                len = g.row_len[u];
                rp = g.row_ptr[u];
                if (len <= a.small_max) bucket = 0;
                else if (len <= a.med_max) bucket = 1;
                else { bucket = 2; nch = (len + a.chunk - 1) / a.chunk; }
            }
            const unsigned bf = __ballot_sync(kFull, leader && node_in);
            if (bf == 0) continue;
            const unsigned bs = __ballot_sync(kFull, bucket == 0);
            const unsigned bm = __ballot_sync(kFull, bucket == 1);
            int lch = (bucket == 2) ? nch : 0;
            int sc = lch;  // inclusive warp scan of chunk counts
    #pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(kFull, sc, o);
                if (lane >= o) sc += y;
            }
            const int wch = __shfl_sync(kFull, sc, 31);
            int b0 = 0, b1 = 0, b2 = 0, b3 = 0;
            if (lane == 0) {
                b0 = atomicAdd(&ts.front_cnt[par], __popc(bf));
                if (bs) b1 = atomicAdd(&ts.small_cnt[par], __popc(bs));
                if (bm) b2 = atomicAdd(&ts.med_cnt[par], __popc(bm));
                if (wch) b3 = atomicAdd(&ts.large_cnt[par], wch);
            }
            b0 = __shfl_sync(kFull, b0, 0);
            b1 = __shfl_sync(kFull, b1, 0);
            b2 = __shfl_sync(kFull, b2, 0);
            b3 = __shfl_sync(kFull, b3, 0);
            const unsigned below = (1u << lane) - 1u;
            int fidx = 0;
            if (leader && node_in) {
                fidx = b0 + __popc(bf & below);
                PushItem item;
                item.rp = rp;
                item.len = len;
                item.fidx = fidx;
                if (bucket == 0) bsmall[b1 + __popc(bs & below)] = item;
                else if (bucket == 1) bmed_end[-(b2 + __popc(bm & below))] = item;
                else {
                    int lb = b3 + (sc - lch);
                    for (int ch = 0; ch < nch; ++ch) {
                        item.rp = rp + (long long)ch * a.chunk;
                        item.len = min(a.chunk, len - ch * a.chunk);
                        blarge[lb + ch] = item;
                    }
                }
                my_vol += du;
                my_cnt += 1;
            }
            fidx = __shfl_sync(kFull, fidx, grp_w * L);
            if (node_in) vstore<T, VEC>(Pw + (int64_t)fidx * W + c0, push);
        }
    }
    // ---- flush per-column counters (one global atomic per column per block) ----
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
        atomicAdd(&ps.acc_col_nodes, (unsigned long long)ps.col_nodes[threadIdx.x]);
        atomicAdd(&ps.acc_col_vol, ps.col_oper[threadIdx.x]);
    }
    if (threadIdx.x == 0 && ps.nodes) {
        atomicAdd(&ts.union_vol[par], ps.vol);
        ps.acc_union_nodes += (unsigned long long)ps.nodes;
        ps.acc_union_vol += ps.vol;
    }
    __syncthreads();
}

// Zero the counters a tile's next round will fill (block 0, before PREP
// work; these fields were last used a round ago, see gde_common.cuh).
template <int W>
__device__ void zero_next_counters(const PushArgs& a, int t, int level) {
    TileState& ts = a.ts[t];
    const int np = (level & 1) ^ 1;
    if (threadIdx.x == 0) {
        ts.cand_cnt[(level + 2) % 3] = 0;
        ts.front_cnt[np] = 0;
        ts.small_cnt[np] = 0;
        ts.med_cnt[np] = 0;
        ts.large_cnt[np] = 0;
        ts.union_vol[np] = 0.0;
    }
    if (threadIdx.x < W) {
        ColState& c = a.cs[(int64_t)t * W + threadIdx.x];
        c.round_active[np] = 0;
        c.check_cnt[np] = 0;
        if (a.tp[t].method == M_HK_GLOBAL && hk_relaxed(a.tp[t])) {
            c.sweep_sum += max(1, c.hk_sweeps[np ^ 1]);  // this level's sweeps, final after the CHECK phase
            c.hk_sweeps[np] = 0;
        }
    }
}

// ---------------------------------------------------------------------------
// SCATTER pieces (tile t, its scatter flags and level)
// ---------------------------------------------------------------------------
template <typename T, int W>
struct ScatterCtx {
    T* tgt;
    int tld;                // row stride of tgt (the solution slab may interleave {x, c})
    const T* Pw;
    int32_t* mark;
    int32_t* next;
    int* next_cnt;
    int stamp;
    bool track;
    bool tgt_scale;
    bool cross;
    const ColState* cs;     // the tile's column states (thresholds for crossing)
    double* rh;             // FP64 residual of the hub prefix (ids < rh_cut), or nullptr
    int rh_cut;
};

template <typename T, int W>
__device__ __forceinline__ ScatterCtx<T, W> scatter_ctx(const PushArgs& a, int t, int level, unsigned char flags) {
    ScatterCtx<T, W> c;
    const int64_t n = a.g.n;
    const int par = level & 1;
    if (flags & SF_HK) {
        // the heat kernel's last level pushes straight into the solution
        if (flags & SF_FINAL) {
            c.tgt = xslab_ptr<T>(a.X, a, t);
            c.tld = (int)x_ld(a);
        } else {
            c.tgt = slab_ptr<T>((level & 1) ? a.R : a.R2, a, t);
            c.tld = a.ld;
        }
    } else {
        c.tgt = slab_ptr<T>(a.R, a, t);
        c.tld = a.ld;
    }
    c.Pw = reinterpret_cast<const T*>(a.P) + (int64_t)t * n * W;
    c.mark = a.mark + (int64_t)t * n;
    c.next = a.cand + ((int64_t)t * 2 + (par ^ 1)) * n;
    c.next_cnt = &a.ts[t].cand_cnt[(level + 1) % 3];
    c.stamp = a.ts[t].stamp + level + 1;
    c.track = (flags & SF_TRACK) != 0;
    c.tgt_scale = (flags & SF_TGTSCALE) != 0;
    c.cross = (flags & SF_CROSS) != 0;
    c.cs = a.cs + (int64_t)t * W;
    c.rh = (sizeof(T) == 4 && W == 1 && c.cross) ? rh_ptr(a, t) : nullptr;
    c.rh_cut = a.rh_cut;
    return c;
}

template <typename T, int VEC>
__device__ __forceinline__ void push_edge(const DevGraph& g, T* tgt, int64_t ld, int c0, int v, const Vec<T, VEC>& p,
                                          bool tgt_scale);

// Did an addition take node v's residual from `old` to `s` across its
// threshold theta * d_v?  Exact; FP32 residuals on integer degrees decide in
// FP32 outside the band of ge_threshold.
template <typename T>
__device__ __forceinline__ bool crossed(const DevGraph& g, int v, T old, T s, double theta, float theta_f) {
    if constexpr (sizeof(T) == 4) {
        if (g.degf_exact) {
            const float df = g.degf[v];
            const float t32 = theta_f * df;
            return !ge_threshold((float)old, t32, theta, (double)df) && ge_threshold((float)s, t32, theta, (double)df);
        }
    }
    const double thr = theta * (g.degf_exact ? (double)g.degf[v] : g.degd[v]);
    return ((double)old < thr) && ((double)s >= thr);
}

template <typename T, int VEC>
__device__ __forceinline__ void load_thetas(const ColState* cs, int c0, bool cross, double (&theta)[VEC],
                                            float (&theta_f)[VEC]) {
#pragma unroll
    for (int k = 0; k < VEC; ++k) {
        theta[k] = cross ? cs[c0 + k].theta : 0.0;
        theta_f[k] = (float)theta[k];
    }
}

// One edge of a push for the L lanes of a group: add p into row v of the
// target; then either append v on a threshold crossing (SF_CROSS) or append
// every touched v (sparse tracking).  Every lane of the warp must call it.
template <typename T, int W, int VEC, int L>
__device__ __forceinline__ void edge_step(const PushArgs& a, const ScatterCtx<T, W>& c, bool ok, int v, int c0,
                                          int lane_g, int grp_w, const Vec<T, VEC>& p, const double (&theta)[VEC],
                                          const float (&theta_f)[VEC]) {
    bool cr = false;
    bool combined = false;
    if constexpr (VEC == 1 && L == 1) {
        // Hubs (degree-sorted prefix) receive pushes from many frontier leaves
        // in the same round; lanes of a warp that target the same hub add in
        // shared memory first and one lane issues the global atomic.  The
        // crossing test on the combined add is the same test on the stored
        // value (all additions are non-negative).
        if (!c.tgt_scale) {
            const bool hub = ok && v < a.g.hub_cut;
            if (__any_sync(kFull, hub)) {
                const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
                const unsigned peers = __match_any_sync(kFull, hub ? v : -1 - lane);
                const int leader = __ffs(peers) - 1;
                __shared__ T agg[kWarps][32];
                if (hub && lane == leader) agg[warp][lane] = T(0);
                __syncwarp();
                if (hub) atomicAdd(&agg[warp][leader], p.v[0]);
                __syncwarp();
                if (hub && lane == leader) {
                    const T tot = agg[warp][lane];
                    T* addr = c.tgt + (int64_t)v * c.tld;
                    if (c.cross) {
                        const T old = atomicAdd(addr, tot);
                        const T s = old + tot;
                        cr = crossed<T>(a.g, v, old, s, theta[0], theta_f[0]);
                    } else {
                        atomicAdd(addr, tot);
                    }
                }
                __syncwarp();
                combined = hub;
            }
        }
    }
    if (ok && !combined) {
        if (c.cross) {
            Vec<T, VEC> old;
            vatomic_ret<T, VEC>(c.tgt + (int64_t)v * c.tld + c0, p, old);
#pragma unroll
            for (int k = 0; k < VEC; ++k) {
                if (p.v[k] == T(0)) continue;
                const T s = old.v[k] + p.v[k];  // the value the atomic stored
                cr |= crossed<T>(a.g, v, old.v[k], s, theta[k], theta_f[k]);
            }
        } else {
            push_edge<T, VEC>(a.g, c.tgt, c.tld, c0, v, p, c.tgt_scale);
        }
    }
    if (c.cross) {
        const unsigned b = __ballot_sync(kFull, cr);
        const unsigned gm = ((L == 32) ? kFull : ((1u << L) - 1u)) << (grp_w * L);
        append_once(ok && lane_g == 0 && (b & gm) != 0, v, c.mark, c.stamp, c.next, c.next_cnt, kFull);
    } else if (c.track) {
        append_once(ok && lane_g == 0, v, c.mark, c.stamp, c.next, c.next_cnt, kFull);
    }
}

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

// Medium rows and chunks of long rows: one warp per work item, items
// [beg, end) of `items` read with stride `step` (+1 for chunks, -1 for
// medium rows, which fill the short-row array from its end; each item is at most a.med_max / a.chunk edges, a
// few dependent warp iterations, so no hub row becomes the round's critical
// path).  The item carries the row's start and length, so the warp goes
// straight from the item to the column indices.
template <typename T, int W>
__device__ void scatter_warp_items(const PushArgs& a, const PushItem* items, int step,
                                   const ScatterCtx<T, W>& c, long long beg, long long end) {
    constexpr int VEC = (sizeof(T) == 4) ? (W >= 4 ? 4 : W) : (W >= 2 ? 2 : 1);
    constexpr int L = W / VEC;
    constexpr int GPW = 32 / L;
    const DevGraph& g = a.g;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lane_g = lane % L, grp_w = lane / L;
    const int c0 = lane_g * VEC;
    double theta[VEC];
    float theta_f[VEC];
    load_thetas<T, VEC>(c.cs, c0, c.cross, theta, theta_f);
    for (long long k = beg + warp; k < end; k += kWarps) {
        const PushItem it = items[k * step];
        Vec<T, VEC> p;
        vload<T, VEC>(c.Pw + (int64_t)it.fidx * W + c0, p);
        for (int j0 = 0; j0 < it.len; j0 += GPW) {
            const int j = j0 + grp_w;
            const bool ok = j < it.len;
            const int v = ok ? g.col[it.rp + j] : 0;
            edge_step<T, W, VEC, L>(a, c, ok, v, c0, lane_g, grp_w, p, theta, theta_f);
        }
    }
}

// ---------------------------------------------------------------------------
// Single-column tiles (W = 1: served queries, single-column feature pushes).
// Each lane keeps kEdgeILP independent edges in flight -- column loads, then
// residual atomics, then threshold tests -- instead of one dependent chain
// per edge: the kernel is bound by memory latency, not bandwidth.
// ---------------------------------------------------------------------------
constexpr int kEdgeILP = GDE_EDGE_ILP;

// Warp-aggregated append of up to kEdgeILP crossing targets per lane (one
// global atomic per warp).  On a W = 1 crossing tile every node crosses its
// threshold at most once per round (additions are non-negative and every
// residual starts the round below threshold), so no dedup mark is needed.
__device__ __forceinline__ void append_crossings(const bool (&cr)[kEdgeILP], const int (&v)[kEdgeILP], int32_t* list,
                                                 int* cnt) {
    int mine = 0;
#pragma unroll
    for (int u = 0; u < kEdgeILP; ++u) mine += cr[u] ? 1 : 0;
    if (__ballot_sync(kFull, mine != 0) == 0) return;
    const int lane = threadIdx.x & 31;
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(kFull, incl, 31);
    int base = 0;
    if (lane == 0) base = atomicAdd(cnt, total);
    int pos = __shfl_sync(kFull, base, 0) + incl - mine;
#pragma unroll
    for (int u = 0; u < kEdgeILP; ++u)
        if (cr[u]) list[pos++] = v[u];
}

// Push value p along kEdgeILP edges per lane (targets v[u] where ok[u]);
// `hub_ok[u]` marks edges already added through the warp's hub combine
// (their crossing result is in hub_cr[u]).
template <typename T>
__device__ __forceinline__ void edges_w1(const PushArgs& a, const ScatterCtx<T, 1>& c, const bool (&ok)[kEdgeILP],
                                         const int (&v)[kEdgeILP], const uint32_t (&dcode)[kEdgeILP],
                                         const T (&p)[kEdgeILP], double theta, const bool (&hub_done)[kEdgeILP],
                                         const bool (&hub_cr)[kEdgeILP]) {
    const DevGraph& g = a.g;
    if (c.cross) {
        const float theta_f = (float)theta;
        bool glob[kEdgeILP];
#pragma unroll
        for (int u = 0; u < kEdgeILP; ++u) glob[u] = ok[u] && !hub_done[u];
        float df[kEdgeILP];
        T old[kEdgeILP];
#pragma unroll
        for (int u = 0; u < kEdgeILP; ++u) {
            df[u] = 1.f;
            if (glob[u]) df[u] = (dcode[u] != g.deg_esc) ? (float)dcode[u] : g.degf[v[u]];
        }
        bool hd[kEdgeILP];     // target in the FP64 hub prefix
        double oldd[kEdgeILP];
#pragma unroll
        for (int u = 0; u < kEdgeILP; ++u) {
            hd[u] = c.rh && glob[u] && v[u] < c.rh_cut;
            oldd[u] = 0.0;
            old[u] = T(0);
            if (hd[u]) oldd[u] = atomicAdd(c.rh + v[u], (double)p[u]);
            else if (glob[u]) old[u] = atomicAdd(c.tgt + (int64_t)v[u] * c.tld, p[u]);
        }
        bool cr[kEdgeILP];
#pragma unroll
        for (int u = 0; u < kEdgeILP; ++u) {
            cr[u] = hub_cr[u];
            if (hd[u]) {
                const double dv = g.degf_exact ? (double)df[u] : g.degd[v[u]];
                const double thr = theta * dv;
                cr[u] = (oldd[u] < thr) && (oldd[u] + (double)p[u] >= thr);  // the value the atomic stored
            } else if (glob[u]) {
                const T s = old[u] + p[u];  // the value the atomic stored
                if constexpr (sizeof(T) == 4) {
                    if (g.degf_exact) {
                        const float t32 = theta_f * df[u];
                        cr[u] = !ge_threshold(old[u], t32, theta, (double)df[u]) &&
                                ge_threshold(s, t32, theta, (double)df[u]);
                        continue;
                    }
                }
                const double dv = g.degf_exact ? (double)df[u] : g.degd[v[u]];
                const double thr = theta * dv;
                cr[u] = ((double)old[u] < thr) && ((double)s >= thr);
            }
        }
        append_crossings(cr, v, c.next, c.next_cnt);
    } else {
#pragma unroll
        for (int u = 0; u < kEdgeILP; ++u) {
            if (!ok[u] || hub_done[u] || p[u] == T(0)) continue;
            T q = p[u];
            if (c.tgt_scale) q = q / ((sizeof(T) == 4) ? (T)g.tfac_f[v[u]] : (T)g.tfac[v[u]]);  // InstantGNN.py:31
            atomicAdd(c.tgt + (int64_t)v[u] * c.tld, q);
        }
        if (c.track) {
#pragma unroll
            for (int u = 0; u < kEdgeILP; ++u) append_once(ok[u], v[u], c.mark, c.stamp, c.next, c.next_cnt, kFull);
        }
    }
}

// Target id and degree code of edge position j (code == deg_esc: read degf).
__device__ __forceinline__ void load_edge(const DevGraph& g, long long j, int& v, uint32_t& dcode) {
    if (g.col_deg) {
        const uint32_t w = g.col_deg[j];
        v = (int)(w & ((1u << g.idx_bits) - 1u));
        dcode = w >> g.idx_bits;
    } else {
        v = g.col[j];
        dcode = g.deg_esc;
    }
}

// W = 1 medium rows and long-row chunks: one warp per item, 32 * kEdgeILP
// edges per warp iteration.  Lanes of one item target distinct nodes, so no
// hub combine applies here.
template <typename T>
__device__ void scatter_warp_items_w1(const PushArgs& a, const PushItem* items, int step, const ScatterCtx<T, 1>& c,
                                      long long beg, long long end) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double theta = c.cross ? c.cs[0].theta : 0.0;
    bool none[kEdgeILP];
#pragma unroll
    for (int u = 0; u < kEdgeILP; ++u) none[u] = false;
    for (long long k = beg + warp; k < end; k += kWarps) {
        const PushItem it = items[k * step];
        const T pv = c.Pw[it.fidx];
        T p[kEdgeILP];
#pragma unroll
        for (int u = 0; u < kEdgeILP; ++u) p[u] = pv;
#if GDE_VEC_COLS
        // 128-bit column loads: the row's first 16-byte boundary, then each
        // lane takes 4 consecutive column words with one load and pushes them
        // kEdgeILP at a time
        static_assert(4 % kEdgeILP == 0, "4 column words per lane split into kEdgeILP-edge steps");
        if (a.g.col_deg && it.len >= 128) {
            const int head = (int)((4 - (it.rp & 3)) & 3);
            {
                bool ok[kEdgeILP];
                int v[kEdgeILP];
                uint32_t dc[kEdgeILP];
#pragma unroll
                for (int u = 0; u < kEdgeILP; ++u) {
                    ok[u] = (u == 0) && lane < head;
                    v[u] = 0;
                    dc[u] = 0;
                    if (ok[u]) load_edge(a.g, it.rp + lane, v[u], dc[u]);
                }
                edges_w1<T>(a, c, ok, v, dc, p, theta, none, none);
            }
            const uint32_t* body = a.g.col_deg + it.rp + head;  // 16-byte aligned
            const int nb = it.len - head;
            const uint32_t mask = (1u << a.g.idx_bits) - 1u;
            for (int b0 = 0; b0 < nb; b0 += 128) {
                const int e = b0 + 4 * lane;
                uint32_t w[4] = {0u, 0u, 0u, 0u};
                if (e + 3 < nb) {
                    const uint4 q = *reinterpret_cast<const uint4*>(body + e);
                    w[0] = q.x; w[1] = q.y; w[2] = q.z; w[3] = q.w;
                } else {
#pragma unroll
                    for (int i = 0; i < 4; ++i)
                        if (e + i < nb) w[i] = body[e + i];
                }
#pragma unroll
                for (int h = 0; h < 4; h += kEdgeILP) {
                    bool ok[kEdgeILP];
                    int v[kEdgeILP];
                    uint32_t dc[kEdgeILP];
#pragma unroll
                    for (int u = 0; u < kEdgeILP; ++u) {
                        ok[u] = e + h + u < nb;
                        v[u] = (int)(w[h + u] & mask);
                        dc[u] = w[h + u] >> a.g.idx_bits;
                    }
                    edges_w1<T>(a, c, ok, v, dc, p, theta, none, none);
                }
            }
            continue;
        }
#endif
        for (int j0 = 0; j0 < it.len; j0 += 32 * kEdgeILP) {
            bool ok[kEdgeILP];
            int v[kEdgeILP];
            uint32_t dc[kEdgeILP];
#pragma unroll
            for (int u = 0; u < kEdgeILP; ++u) {
                const int j = j0 + u * 32 + lane;
                ok[u] = j < it.len;
                v[u] = 0;
                dc[u] = 0;
                if (ok[u]) load_edge(a.g, it.rp + j, v[u], dc[u]);
            }
            edges_w1<T>(a, c, ok, v, dc, p, theta, none, none);
        }
    }
}

// W = 1 short rows flattened per warp: a warp takes GROUP consecutive items
// and spreads their edges evenly over its lanes, 32 * kEdgeILP edges per
// step (the lane holding edge e finds its row by a binary search over the
// warp's exclusive edge offsets), so a step carries every row's edges
// instead of one row per lane.  Lanes of a step whose edges hit the same hub
// (degree-sorted prefix) add in shared memory first and one lane issues the
// global atomic; the crossing test on the combined add is the same test on
// the stored value.  (Flattening medium rows the same way measured slower
// than a warp per medium row.)
template <typename T, int GROUP>
__device__ void scatter_flat_w1(const PushArgs& a, const PushItem* items, int step, const ScatterCtx<T, 1>& c,
                                long long beg, long long end) {
    const DevGraph& g = a.g;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double theta = c.cross ? c.cs[0].theta : 0.0;
    __shared__ T fagg[kWarps][32];
    __shared__ double faggd[kWarps][32];  // hub-prefix targets: the warp's sum in FP64
    for (long long kb = beg + (long long)warp * GROUP; kb < end; kb += (long long)kWarps * GROUP) {
        const long long k = kb + lane;
        int len = 0;
        long long rp = 0;
        T pv = T(0);
        if (lane < GROUP && k < end) {
            const PushItem it = items[k * step];
            rp = it.rp;
            len = it.len;
            pv = c.Pw[it.fidx];
        }
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        const int excl = incl - len;
        for (int e0 = 0; e0 < total; e0 += 32 * kEdgeILP) {
            bool ok[kEdgeILP], hub_done[kEdgeILP], hub_cr[kEdgeILP];
            int v[kEdgeILP];
            uint32_t dc[kEdgeILP];
            T p[kEdgeILP];
#pragma unroll
            for (int u = 0; u < kEdgeILP; ++u) {
                const int e = e0 + u * 32 + lane;
                ok[u] = e < total;
                // the row holding edge e: the last lane whose offset is <= e
                int r = 0;
#pragma unroll
                for (int b = 16; b > 0; b >>= 1) {
                    const int ex = __shfl_sync(kFull, excl, (r + b) & 31);
                    if (r + b < GROUP && ex <= e) r += b;
                }
                const long long rpr = __shfl_sync(kFull, rp, r);
                const int exr = __shfl_sync(kFull, excl, r);
                p[u] = __shfl_sync(kFull, pv, r);
                v[u] = 0;
                dc[u] = 0;
                if (ok[u]) load_edge(g, rpr + (e - exr), v[u], dc[u]);
                hub_done[u] = false;
                hub_cr[u] = false;
            }
            if (!c.tgt_scale) {
#pragma unroll
                for (int u = 0; u < kEdgeILP; ++u) {
                    const bool hub = ok[u] && v[u] < g.hub_cut;
                    if (!__any_sync(kFull, hub)) continue;
                    const unsigned peers = __match_any_sync(kFull, hub ? v[u] : -1 - lane);
                    const int leader = __ffs(peers) - 1;
                    const bool hd = hub && c.rh && v[u] < c.rh_cut;
                    if (hub && lane == leader) {
                        fagg[warp][lane] = T(0);
                        faggd[warp][lane] = 0.0;
                    }
                    __syncwarp();
                    if (hd) atomicAdd(&faggd[warp][leader], (double)p[u]);
                    else if (hub) atomicAdd(&fagg[warp][leader], p[u]);
                    __syncwarp();
                    if (hd && lane == leader) {
                        // FP64 hub prefix: the combined add and the crossing test in FP64
                        const double tot = faggd[warp][lane];
                        const double old = atomicAdd(c.rh + v[u], tot);
                        const double dv = (dc[u] != g.deg_esc) ? (double)dc[u]
                                          : (g.degf_exact ? (double)g.degf[v[u]] : g.degd[v[u]]);
                        const double thr = theta * dv;
                        hub_cr[u] = (old < thr) && (old + tot >= thr);
                    } else if (hub && lane == leader) {
                        const T tot = fagg[warp][lane];
                        T* addr = c.tgt + (int64_t)v[u] * c.tld;
                        if (c.cross) {
                            const T old = atomicAdd(addr, tot);
                            const T s = old + tot;
                            const double dv = (dc[u] != g.deg_esc) ? (double)dc[u]
                                              : (g.degf_exact ? (double)g.degf[v[u]] : g.degd[v[u]]);
                            if constexpr (sizeof(T) == 4) {
                                if (g.degf_exact) {
                                    const float t32 = (float)theta * (float)dv;
                                    hub_cr[u] = !ge_threshold(old, t32, theta, dv) && ge_threshold(s, t32, theta, dv);
                                } else {
                                    hub_cr[u] = ((double)old < theta * dv) && ((double)s >= theta * dv);
                                }
                            } else {
                                const double thr = theta * dv;
                                hub_cr[u] = ((double)old < thr) && ((double)s >= thr);
                            }
                        } else {
                            atomicAdd(addr, tot);
                        }
                    }
                    __syncwarp();
                    hub_done[u] = hub;
                }
            }
            edges_w1<T>(a, c, ok, v, dc, p, theta, hub_done, hub_cr);
        }
    }
}

// Short rows of a W > 1 tile (a lane group of L = W / VEC lanes moves a
// row's W columns as VEC-wide vector atomics), flattened per warp: the
// warp's GPW rows spread their edges over its GPW groups, one edge per group
// per step (the group holding edge e finds its row by a binary search over
// the groups' edge offsets), instead of one row per group and as many steps
// as the warp's longest row (+4% on the 8-column InstantGNN push).
template <typename T, int W>
__device__ void scatter_small_flat(const PushArgs& a, int t, const ScatterCtx<T, W>& c, long long beg,
                                   long long end) {
    constexpr int VEC = (sizeof(T) == 4) ? (W >= 4 ? 4 : W) : (W >= 2 ? 2 : 1);
    constexpr int L = W / VEC;
    constexpr int GPW = 32 / L;
    const DevGraph& g = a.g;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lane_g = lane % L, grp_w = lane / L;
    const int c0 = lane_g * VEC;
    const PushItem* bsmall = a.bsmall + (int64_t)t * a.g.n;
    double theta[VEC];
    float theta_f[VEC];
    load_thetas<T, VEC>(c.cs, c0, c.cross, theta, theta_f);
    for (long long kb = beg + (long long)warp * GPW; kb < end; kb += (long long)kWarps * GPW) {
        const long long k = kb + grp_w;
        int len = 0;
        long long rp = 0;
        Vec<T, VEC> p;
#pragma unroll
        for (int i = 0; i < VEC; ++i) p.v[i] = T(0);
        if (k < end) {
            const PushItem it = bsmall[k];
            rp = it.rp;
            len = it.len;
            vload<T, VEC>(c.Pw + (int64_t)it.fidx * W + c0, p);
        }
        // edge offsets by group: each group's first lane carries its row length
        int incl = (lane_g == 0) ? len : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        const int excl = incl - ((lane_g == 0) ? len : 0);  // valid on each group's first lane
        for (int e0 = 0; e0 < total; e0 += GPW) {
            const int e = e0 + grp_w;
            const bool ok = e < total;
            // the group holding edge e: the last group whose offset is <= e
            int r = 0;
#pragma unroll
            for (int b = GPW / 2; b > 0; b >>= 1) {
                const int ex = __shfl_sync(kFull, excl, ((r + b) * L) & 31);
                if (r + b < GPW && ex <= e) r += b;
            }
            const long long rpr = __shfl_sync(kFull, rp, r * L);
            const int exr = __shfl_sync(kFull, excl, r * L);
            Vec<T, VEC> pr;
#pragma unroll
            for (int i = 0; i < VEC; ++i) pr.v[i] = __shfl_sync(kFull, p.v[i], r * L + lane_g);
            const int v = ok ? g.col[rpr + (e - exr)] : 0;
            edge_step<T, W, VEC, L>(a, c, ok, v, c0, lane_g, grp_w, pr, theta, theta_f);
        }
    }
}

// HK: drop this level's sub-threshold residuals (hk_solver.py:284); the
// frontier's own entries were already moved into x.
template <typename T, int W>
__device__ void hk_drop(const PushArgs& a, int t, int level, bool dense, int cand_cnt, const GroupInfo& gi) {
    const int64_t n = a.g.n;
    T* Rcur = slab_ptr<T>((level & 1) ? a.R2 : a.R, a, t);
    const int64_t stride = (int64_t)gi.dim * kThreads;
    if (dense) {
        for (int64_t u = (int64_t)gi.blk * kThreads + threadIdx.x; u < n; u += stride)
            for (int c = 0; c < W; ++c) Rcur[u * a.ld + c] = T(0);
    } else {
        const int32_t* cand = a.cand + ((int64_t)t * 2 + (level & 1)) * n;
        for (int64_t i = (int64_t)gi.blk * kThreads + threadIdx.x; i < cand_cnt; i += stride) {
            const int u = cand[i];
            for (int c = 0; c < W; ++c) Rcur[(int64_t)u * a.ld + c] = T(0);
        }
    }
}

// Round bookkeeping for tile t by block 0 (fields read only at the next
// round's start): a local column with no active node this round is finished
// (ppr_solver.py:266-267); a global column whose CHECK found nothing above
// threshold is finished (:292-293); HK stops after its last level
// (hk_solver.py:235); a tile is done when its frontier is empty.
__device__ __forceinline__ bool hk_end_level(const TileParams& tp, int level) {
    const int m = tp.method;
    return method_is_hk(m) && ((m == M_HK_TAYLOR) ? (level >= tp.n_levels) : (level + 1 >= tp.n_levels));
}

// Column part of the bookkeeping: one thread per (live tile, column).
template <int W>
__device__ void finish_columns_all(const PushArgs& a, const RoundSh& rs, int ntl) {
    for (int idx = threadIdx.x; idx < ntl * W; idx += kThreads) {
        const int k = idx / W, c = idx % W;
        const int t = rs.tiles[k];
        const int level = rs.level[k];
        const TileParams& tp = a.tp[t];
        if (c >= tp.ncols) continue;
        const int m = tp.method;
        const int par = level & 1;
        const bool gcheck = (m == M_GLOBAL_GD || m == M_GLOBAL_CHEBY);
        ColState& cs = a.cs[(int64_t)t * W + c];
        if (cs.live) {
            bool worked = gcheck ? (cs.check_cnt[par] > 0) : (cs.round_active[par] > 0);
            if (method_is_hk(m) && m != M_HK_LOCAL) worked = true;  // fixed sweeps per level
            if (worked) cs.rounds += 1;
            if (!worked || hk_end_level(tp, level)) {
                cs.live = 0;
                cs.finish_ns = globaltimer_ns();
            }
        }
    }
}

// Tile part of the bookkeeping (after the column part): one thread per tile.
template <int W>
__device__ void finish_round(const PushArgs& a, int t, int level, bool dense_next) {
    const TileParams& tp = a.tp[t];
    const int par = level & 1;
    const bool hk_end = hk_end_level(tp, level);
    {
        TileState& ts = a.ts[t];
        ts.dense_next[par ^ 1] = dense_next ? 1 : 0;
        // a served heat-kernel slot ends one (empty) round after its last
        // level: that level pushes into x during SCATTER, so x is read out by
        // the next round's retire
        if (ts.front_cnt[par] == 0 || (hk_end && !a.serve)) {
            if (a.serve && a.queue.online) {
                // online slot: its row is gathered by every block of its group
                // in this SCATTER; next round clears the slot and publishes the result
                const ColState& cs = a.cs[(int64_t)t * W];
                OnlineSlot& os = a.queue.slot[t];
                os.oper = cs.oper;
                os.rounds = cs.rounds;
                os.finish_ns = globaltimer_ns();
                ts.done = SLOT_DRAIN;
            } else if (a.serve) {
                // served slot: the query's result is extracted and the slot
                // cleared by every block of its group in this SCATTER; admit next round
                const ColState& cs = a.cs[(int64_t)t * W];
                const int q = ts.qid;
                a.queue.oper[q] = cs.oper;
                a.queue.rounds[q] = cs.rounds;
                a.queue.finish_ns[q] = globaltimer_ns();
                ts.done = SLOT_IDLE;
            } else {
                ts.done = SLOT_DONE;
            }
        }
        atomicAdd(&a.stats->rounds, 1ull);
        if (dense_next) atomicAdd(&a.stats->dense_rounds, 1ull);
    }
}

// Served solves: block 0 puts the next queued query into an idle slot (the
// slot's vectors were cleared when its previous query retired, a round ago).
// Everything written here is read only from the next round on.
template <typename T, int W>
__device__ void admit_query(const PushArgs& a, int t, int it) {
    if (threadIdx.x != 0) return;
    TileState& ts = a.ts[t];
    const ServeQueue& q = a.queue;
    // Queries a hash-table block gave back come first (they arrived before
    // the dense-class queries still queued), then the next query in order
    // (the dense-class order when small queries go to the hash-table blocks).
    // Group leaders take queries concurrently.
    const unsigned long long now = globaltimer_ns();
    int qid = -1;
    int sp_left = 0;
    if (q.sp_blocks > 0) {
        // sp_left is read first: at zero every ovf position has been handed out
        sp_left = ld_acquire_gpu_i(q.sp_left);
        for (int tries = 0; tries < 4096 && qid < 0; ++tries) {
            const int c = ld_volatile_i(q.ovf_next);
            if (c >= ld_volatile_i(q.ovf_cnt)) break;
            if (atomicCAS(q.ovf_next, c, c + 1) == c) {
                // the position is handed out before its id is stored: wait for it (bounded)
                int v = ld_volatile_i(&q.ovf[c]);
                for (unsigned long long k = 0; v < 0; ++k) {
                    if (k > (a.spin_limit ? a.spin_limit : (1ull << 26))) {
                        atomicCAS(a.err, 0, GDE_EHANG);
                        return;
                    }
                    v = ld_volatile_i(&q.ovf[c]);
                }
                qid = v;
            }
        }
    }
    bool dense_left = true;
    const int nd = q.order_d ? q.nd : q.nq;
    if (qid < 0 && q.arrival_ns) {
        // block 0 stamps the launch start; other groups may get here first
        const unsigned long long st0 = *(volatile const unsigned long long*)&a.stats->start_ns;
        if (st0 == 0) return;
        for (int tries = 0; tries < 4096; ++tries) {
            const int c = ld_volatile_i(q.next);
            if (c >= nd) {
                dense_left = false;
                break;
            }
            const int cq = q.order_d ? q.order_d[c] : c;
            if (now < st0 + (unsigned long long)q.arrival_ns[cq]) return;  // not arrived yet
            if (atomicCAS(q.next, c, c + 1) == c) {
                qid = cq;
                break;
            }
        }
    } else if (qid < 0) {
        const int c = atomicAdd(q.next, 1);
        if (c < nd) qid = q.order_d ? q.order_d[c] : c;
        else dense_left = false;
    }
    if (qid < 0) {
        // nothing now; the slot is done when the dense order is used up and
        // no hash-table query is left to give one back
        if (!dense_left &&
            (q.sp_blocks == 0 || (sp_left == 0 && ld_volatile_i(q.ovf_next) >= ld_volatile_i(q.ovf_cnt))))
            ts.done = SLOT_EMPTY;
        return;
    }
    const int64_t n = a.g.n;
    const int seed = q.seed[qid];
    // stamps must keep growing within the slot: skip past the last query's
    ts.stamp = ts.stamp + (it - ts.t0) + 2;
    for (int i = 0; i < 3; ++i) ts.cand_cnt[i] = 0;
    for (int i = 0; i < 2; ++i) {
        ts.front_cnt[i] = ts.small_cnt[i] = ts.med_cnt[i] = ts.large_cnt[i] = 0;
        ts.dense_next[i] = 0;
        ts.union_vol[i] = 0.0;
    }
    a.cand[((int64_t)t * 2 + 0) * n] = seed;  // level-0 candidates: the seed
    ts.cand_cnt[0] = 1;
    ts.t0 = it + 1;
    ts.qid = qid;
    if (q.kind) {
        // mixed queue: the slot takes the query's kind and parameters
        TileParams& tp = a.tp[t];
        const int k = q.kind[qid];
        tp.kind = k;
        tp.method = (k == KIND_HK) ? M_HK_LOCAL : M_LOCAL_GD;
        tp.alpha = (k == KIND_HK) ? 0.0 : q.alpha[qid];
        tp.tau = q.tau;
        tp.n_levels = (k == KIND_HK) ? q.n_levels[qid] : 0;
        tp.psi_tab = (k == KIND_HK) ? q.psi + q.psi_off[qid] : nullptr;
    }
    ColState& cs = a.cs[(int64_t)t * W];
    cs.theta = q.theta[qid];
    cs.oper = 0.0;
    cs.fsum = 0;
    cs.live = 1;
    cs.rounds = 0;
    cs.round_active[0] = cs.round_active[1] = 0;
    cs.check_cnt[0] = cs.check_cnt[1] = 0;
    cs.seed = seed;
    cs.finish_ns = 0;
    if (sizeof(T) == 4 && a.RH && tile_crosses(a.tp[t]) && seed < a.rh_cut) rh_ptr(a, t)[seed] = q.r0[qid];
    else slab_ptr<T>(a.R, a, t)[(int64_t)seed * a.ld] = (T)q.r0[qid];
    if (q.start_ns[qid] == 0) q.start_ns[qid] = now;  // an overflowed query keeps its first admission
    __threadfence();
    ts.done = SLOT_LIVE;
}

// Served solves: write a retiring slot's solution row and clear the slot's
// vectors, internal nodes [beg, end).  The row is written in internal node
// order (sequential reads, writes and clears); the host permutes finished
// rows to caller order after the launch (permute_rows_to_caller).
template <typename T, int W>
__device__ void retire_range(const PushArgs& a, int t, long long beg, long long end) {
    const ServeQueue& q = a.queue;
    const int qid = a.ts[t].qid;
    T* X = xslab_ptr<T>(a.X, a, t);
    T* R = slab_ptr<T>(a.R, a, t);
    T* R2 = a.R2 ? slab_ptr<T>(a.R2, a, t) : nullptr;
    float* XC = a.kahan ? xslab_ptr<float>(a.XC, a, t) : nullptr;
    double* rh = (sizeof(T) == 4) ? rh_ptr(a, t) : nullptr;  // FP64 hub prefix
    const int64_t xld = x_ld(a);
    const int si = q.seed[qid];
    const int kind = q.kind ? q.kind[qid] : a.tp[t].kind;
    // Katz GD: xt[s_node] -= 1 (katz_solver.py:243); HK: xt / e^tau (hk_solver.py:295)
    const double seed_add = q.kind ? (kind == KIND_KATZ ? -1.0 : 0.0) : q.seed_add;
    const double xdiv = (kind == KIND_HK) ? q.hk_scale : 1.0;
    const int64_t orow = (int64_t)qid * q.ld_out;
    float* xo32 = (q.x_out && !q.out64) ? reinterpret_cast<float*>(q.x_out) + orow : nullptr;
    double* xo64 = (q.x_out && q.out64) ? reinterpret_cast<double*>(q.x_out) + orow : nullptr;
    // streaming (evict-first) loads and output stores: a retiring row is
    // read and written once and should not push the residual slabs out of L2
    if (a.xq) {
        // the solution stays in the query's own slab (read out after the
        // launch): only the slot's residual is extracted and cleared here
        for (long long v = beg + threadIdx.x; v < end; v += kThreads) {
            const int64_t o = v * a.ld;
            const bool hv = rh && v < a.rh_cut;
            if (q.r_out) {
                const double rv = hv ? rh[v] : (double)R[o];
                if (q.out64) reinterpret_cast<double*>(q.r_out)[orow + v] = rv;
                else reinterpret_cast<float*>(q.r_out)[orow + v] = (float)rv;
            }
            R[o] = T(0);
            if (hv) rh[v] = 0.0;
            if (R2) R2[o] = T(0);
        }
        return;
    }
    for (long long v = beg + threadIdx.x; v < end; v += kThreads) {
        const int64_t o = v * a.ld, xo = v * xld;
        double x = (double)__ldcs(X + xo);
        if (XC) x -= (double)__ldcs(XC + xo);  // Kahan: the sum is X - XC
        if (v == si) x = x + seed_add;
        if (xdiv != 1.0) x = x / xdiv;
        if (xo32) __stcs(xo32 + v, (float)x);
        if (xo64) __stcs(xo64 + v, x);
        const bool hv = rh && v < a.rh_cut;
        if (q.r_out) {
            const double rv = hv ? rh[v] : (double)R[o];
            if (q.out64) reinterpret_cast<double*>(q.r_out)[orow + v] = rv;
            else reinterpret_cast<float*>(q.r_out)[orow + v] = (float)rv;
        }
        X[xo] = T(0);
        R[o] = T(0);
        if (hv) rh[v] = 0.0;
        if (R2) R2[o] = T(0);
        if (XC) XC[xo] = 0.f;
    }
}

// ---------------------------------------------------------------------------
// Online server: the request ring and completion records live in pinned host
// memory.  The host publishes a request by a release store of `tail` after
// writing the entry; the device reads `tail` with an acquire load at system
// scope, then the entry.  A completion record is filled, then published by a
// release store of done_ticket.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long ld_acquire_sys(const long long* p) {
    long long v;
    asm volatile("ld.acquire.sys.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_sys(long long* p, long long v) {
    asm volatile("st.release.sys.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_sys_i(const int* p) {
    int v;
    asm volatile("ld.relaxed.sys.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// The ring reader (thread 0 of group 0's first block, once per round of that
// group): submitted requests go, in ring order, into the mailboxes of idle
// slots of any group; `head` then tells the host that the ring entries are
// free again.  A slot's own group admits the request at its next round end
// (admit_online), so each group keeps its own round count and barrier.
__device__ bool route_online(const PushArgs& a) {
    const ServeQueue& q = a.queue;
    long long head = *q.head;  // only this thread writes it
    const long long tail = ld_acquire_sys(q.tail);
    if (head >= tail) return false;
    const long long head0 = head;
    for (int t = 0; t < a.ntiles && head < tail; ++t) {
        OnlineSlot& os = q.slot[t];
        // the mailbox flag first: an owner that just admitted from it wrote
        // the slot's state before clearing the flag
        if (ld_volatile_i(&os.pending) != 0) continue;
        __threadfence();
        if (ld_volatile_i(&a.ts[t].done) != SLOT_IDLE) continue;
        const volatile OnlineReq* rq = q.req + (head % q.cap);
        OnlineReq m;
        m.kind = rq->kind;
        m.seed = rq->seed;
        m.seed_caller = rq->seed_caller;
        m.n_levels = rq->n_levels;
        m.psi_off = rq->psi_off;
        m.out64 = rq->out64;
        m.theta = rq->theta;
        m.r0 = rq->r0;
        m.alpha = rq->alpha;
        m.x_out = rq->x_out;
        m.ticket = rq->ticket;
        os.mail = m;
        __threadfence();
        *(volatile int*)&os.pending = 1;
        ++head;
    }
    if (head == head0) return false;
    __threadfence_system();
    *q.head = head;
    __threadfence_system();
    return true;
}

// Thread 0 of a group's first block: the request in idle slot t's mailbox
// (placed by route_online) becomes the slot's query from the next round of
// this group on.
template <typename T, int W>
__device__ bool admit_online(const PushArgs& a, int t, int it) {
    const ServeQueue& q = a.queue;
    OnlineSlot& os = q.slot[t];
    if (ld_volatile_i(&os.pending) == 0) return false;
    __threadfence();
    const volatile OnlineReq* rq = &os.mail;
    const int k = rq->kind;
    const int seed = rq->seed;
    os.ticket = rq->ticket;
    os.x_out = rq->x_out;
    os.out64 = rq->out64;
    os.seed_caller = rq->seed_caller;
    os.kind = k;
    os.rounds = 0;
    os.status = GDE_OK;
    os.oper = 0.0;
    os.finish_ns = 0;
    TileState& ts = a.ts[t];
    TileParams& tp = a.tp[t];
    tp.kind = k;
    tp.method = (k == KIND_HK) ? M_HK_LOCAL : M_LOCAL_GD;
    tp.alpha = (k == KIND_HK) ? 0.0 : rq->alpha;
    tp.tau = q.tau;
    tp.n_levels = (k == KIND_HK) ? rq->n_levels : 0;
    tp.psi_tab = (k == KIND_HK) ? q.psi + rq->psi_off : nullptr;
    const double theta = rq->theta, r0 = rq->r0;
    // stamps keep growing within the slot: skip past the last query's
    ts.stamp = ts.stamp + max(it - ts.t0, 0) + 2;
    for (int i = 0; i < 3; ++i) ts.cand_cnt[i] = 0;
    for (int i = 0; i < 2; ++i) {
        ts.front_cnt[i] = ts.small_cnt[i] = ts.med_cnt[i] = ts.large_cnt[i] = 0;
        ts.dense_next[i] = 0;
        ts.union_vol[i] = 0.0;
    }
    const int64_t n = a.g.n;
    a.cand[((int64_t)t * 2 + 0) * n] = seed;  // level-0 candidates: the seed
    ts.cand_cnt[0] = 1;
    ts.t0 = it + 1;
    ts.qid = t;
    ColState& cs = a.cs[(int64_t)t * W];
    cs.theta = theta;
    cs.oper = 0.0;
    cs.fsum = 0;
    cs.live = 1;
    cs.rounds = 0;
    cs.round_active[0] = cs.round_active[1] = 0;
    cs.check_cnt[0] = cs.check_cnt[1] = 0;
    cs.seed = seed;
    cs.finish_ns = 0;
    if (sizeof(T) == 4 && a.RH && tile_crosses(a.tp[t]) && seed < a.rh_cut) rh_ptr(a, t)[seed] = r0;
    else slab_ptr<T>(a.R, a, t)[(int64_t)seed * a.ld] = (T)r0;
    os.admit_ns = globaltimer_ns();
    __threadfence();
    ts.done = SLOT_LIVE;
    __threadfence();
    *(volatile int*)&os.pending = 0;  // after the state: the reader checks the flag first
    return true;
}

// A finished online query's row, caller ids [beg, end): gathered through
// the node permutation into the caller's row, x - c for a Kahan slab, with
// the Katz x[s] -= 1 and the heat kernel's x / e^tau.  Read-only on the
// slot: its vectors are cleared next round, after the gather of every block
// of its group.
template <typename T, int W>
__device__ void gather_online_range(const PushArgs& a, int t, long long beg, long long end) {
    const ServeQueue& q = a.queue;
    const OnlineSlot& os = q.slot[t];
    if (!os.x_out) return;
    const T* X = xslab_ptr<T>(a.X, a, t);
    const float* XC = a.kahan ? xslab_ptr<float>(a.XC, a, t) : nullptr;
    const int64_t xld = x_ld(a);
    const double seed_add = (os.kind == KIND_KATZ) ? -1.0 : 0.0;  // katz_solver.py:243
    const double xdiv = (os.kind == KIND_HK) ? q.hk_scale : 1.0;    // hk_solver.py:295
    for (long long u = beg + threadIdx.x; u < end; u += kThreads) {
        const int64_t v = q.perm ? q.perm[u] : u;
        double x = (double)X[v * xld];
        if (XC) x -= (double)XC[v * xld];
        if (u == os.seed_caller) x += seed_add;
        if (xdiv != 1.0) x /= xdiv;
        if (os.out64) reinterpret_cast<double*>(os.x_out)[u] = x;
        else reinterpret_cast<float*>(os.x_out)[u] = (float)x;
    }
    __threadfence_system();
}

// A drained online slot's vectors back to zero, internal nodes [beg, end).
template <typename T, int W>
__device__ void clear_slot_range(const PushArgs& a, int t, long long beg, long long end) {
    T* X = xslab_ptr<T>(a.X, a, t);
    T* R = slab_ptr<T>(a.R, a, t);
    T* R2 = a.R2 ? slab_ptr<T>(a.R2, a, t) : nullptr;
    float* XC = a.kahan ? xslab_ptr<float>(a.XC, a, t) : nullptr;
    double* rh = (sizeof(T) == 4) ? rh_ptr(a, t) : nullptr;
    const int64_t xld = x_ld(a);
    for (long long v = beg + threadIdx.x; v < end; v += kThreads) {
        R[v * a.ld] = T(0);
        if (rh && v < a.rh_cut) rh[v] = 0.0;
        X[v * xld] = T(0);
        if (XC) XC[v * xld] = 0.f;
        if (R2) R2[v * a.ld] = T(0);
    }
}

// Thread 0 of the slot's group's first block: a drained slot's completion
// record (its row was gathered, by the group's blocks, in the previous round).
__device__ void publish_online(const PushArgs& a, int t) {
    const ServeQueue& q = a.queue;
    const OnlineSlot& os = q.slot[t];
    OnlineDone* d = q.done + (os.ticket % q.cap);
    d->oper = os.oper;
    d->rounds = os.rounds;
    d->status = os.status;
    d->admit_ns = os.admit_ns;
    d->finish_ns = os.finish_ns;
    __threadfence_system();
    st_release_sys(&d->done_ticket, os.ticket);
}

// ---------------------------------------------------------------------------
// Hash-compacted small queries.  One block solves one PPR / Katz local GD
// query at a time with the synchronous rounds of the dense engine (the same
// frontier sets: exact operation counts), but over an open-addressing table
// of sp_cap entries {node id, FP64 residual, FP64 solution} in global memory
// instead of dense n-vectors: a query that touches 10^4 nodes of a 2M-node
// graph keeps 20 B per touched entry (the table stays in the L2) and clears
// only the entries it used.  Rounds meet at __syncthreads, not at a grid
// barrier.  A query that fills 3/4 of the table (or fails a bounded probe)
// is handed to the dense slots and its partial work dropped.
// ---------------------------------------------------------------------------
constexpr int kSpEmpty = -1;
constexpr int kSpProbes = 256;

constexpr int kSpLong = 1024;  // rows at least this long are pushed by the whole block
constexpr int kSpLongMax = 32;

struct SpSh {
    int qid;          // query in hand (-1: none left)
    int cur_cnt, nxt_cnt, used;
    int overflow;
    int rounds;
    double oper;
    unsigned long long col_nodes;
    int nlong;                 // frontier rows of at least kSpLong edges this round
    int long_idx[kSpLongMax];  // their frontier positions
};

__device__ __forceinline__ unsigned sp_hash(int v) { return (unsigned)v * 2654435761u; }

// The entry of node v (inserted with zero residual and solution when new), or
// -1 when the table is full.
__device__ __forceinline__ int sp_find_insert(int32_t* keys, int32_t* used_list, int* used, int cap, int v) {
    const unsigned mask = (unsigned)cap - 1u;
    unsigned h = sp_hash(v) & mask;
    for (int p = 0; p < kSpProbes; ++p) {
        const int k = __ldcg(&keys[h]);
        if (k == v) return (int)h;
        if (k == kSpEmpty) {
            const int prev = atomicCAS(&keys[h], kSpEmpty, v);
            if (prev == kSpEmpty) {
                const int pos = atomicAdd(used, 1);
                if (pos >= (cap >> 2) * 3) return -1;  // load factor 3/4: the query leaves the table
                used_list[pos] = (int)h;
                return (int)h;
            }
            if (prev == v) return (int)h;
        }
        h = (h + 1u) & mask;
    }
    return -1;
}

// One edge push of a hash-table query: find or insert the target, add the
// push value to its FP64 residual, and append it to the next frontier when
// it crosses its threshold (warp-uniform call: every lane of the warp).
__device__ __forceinline__ void sp_push_edge(const DevGraph& g, SpSh& sp, int32_t* keys, int32_t* used_list,
                                             double* R, int32_t* nxt, int cap, double theta, bool act, int64_t e,
                                             double pv) {
    const int lane = threadIdx.x & 31;
    bool cr = false;
    int h = -1;
    if (act && !ld_volatile_i(&sp.overflow)) {
        int v;
        uint32_t dc;
        load_edge(g, e, v, dc);
        h = sp_find_insert(keys, used_list, &sp.used, cap, v);
        if (h < 0) {
            sp.overflow = 1;
        } else {
            const double old = atomicAdd(&R[h], pv);
            const double dv = (dc != g.deg_esc) ? (double)dc : g.degd[v];
            const double thr = theta * dv;
            cr = (old < thr) && (old + pv >= thr);  // ppr_solver.py:284-288
        }
    }
    const unsigned b = __ballot_sync(kFull, cr);
    if (b) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&sp.nxt_cnt, __popc(b));
        base = __shfl_sync(kFull, base, 0);
        if (cr) nxt[base + __popc(b & ((1u << lane) - 1u))] = h;
    }
}

__device__ __noinline__ void sparse_block_loop(const PushArgs& a, int c) {
    __shared__ SpSh sp;
    const ServeQueue& q = a.queue;
    const DevGraph& g = a.g;
    const int cap = q.sp_cap;
    int32_t* keys = q.sp_keys + (int64_t)c * cap;
    double* R = q.sp_r + (int64_t)c * cap;
    double* X = q.sp_x + (int64_t)c * cap;
    int32_t* lists = q.sp_list + (int64_t)c * 3 * cap;
    int32_t* used_list = lists + 2 * cap;
    double* push = q.sp_push + (int64_t)c * cap;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long acc_nodes = 0;
    double acc_vol = 0.0;
    for (;;) {
        // ---- the next small query, in arrival order ----
        if (threadIdx.x == 0) {
            sp.qid = -1;
            for (;;) {
                const int cpos = ld_volatile_i(q.next_s);
                if (cpos >= q.ns) break;
                const int cq = q.order_s[cpos];
                if (q.arrival_ns) {
                    const unsigned long long st0 = *(volatile const unsigned long long*)&a.stats->start_ns;
                    if (st0 == 0 || globaltimer_ns() < st0 + (unsigned long long)q.arrival_ns[cq]) {
                        if (ld_volatile_i(a.err) != 0) break;
                        __nanosleep(2000);  // waits for an arrival time that is finite
                        continue;
                    }
                }
                if (atomicCAS(q.next_s, cpos, cpos + 1) == cpos) {
                    sp.qid = cq;
                    break;
                }
            }
            sp.cur_cnt = 0;
            sp.nxt_cnt = 0;
            sp.used = 0;
            sp.overflow = 0;
            sp.rounds = 0;
            sp.oper = 0.0;
            sp.col_nodes = 0;
        }
        __syncthreads();
        const int qid = sp.qid;
        if (qid < 0) break;
        const int kind = q.kind ? q.kind[qid] : q.kind0;
        const double alpha = q.alpha ? q.alpha[qid] : q.alpha0;
        const double theta = q.theta[qid];
        const int seed = q.seed[qid];
        if (threadIdx.x == 0) {
            q.start_ns[qid] = globaltimer_ns();
            const int h = sp_find_insert(keys, used_list, &sp.used, cap, seed);
            const double r0 = q.r0[qid];
            R[h] = r0;
            lists[0] = h;
            // the seed is the first frontier (ppr_solver.py:237) when at threshold (the assert at :213)
            sp.cur_cnt = (r0 >= theta * g.degd[seed]) ? 1 : 0;
        }
        __syncthreads();
        int par = 0;
        for (int round = 0;; ++round) {
            if (sp.cur_cnt == 0) break;
            if (round >= a.max_rounds) {
                // the round cap: the dense slots run it again and report the cap
                if (threadIdx.x == 0) sp.overflow = 1;
                __syncthreads();
                break;
            }
            int32_t* cur = lists + par * cap;
            int32_t* nxt = lists + (par ^ 1) * cap;
            const int nf = sp.cur_cnt;
            // ---- PREP: move each frontier entry's residual into its solution ----
            double my_oper = 0.0;
            for (int i = threadIdx.x; i < nf; i += kThreads) {
                const int h = cur[i];
                const int u = __ldcg(&keys[h]);
                const double r = __ldcg(&R[h]);
                R[h] = 0.0;
                X[h] += r;
                const double du = g.degd[u];
                push[i] = (kind == KIND_KATZ) ? alpha * r : ((1. - alpha) * r) / du;  // ppr_solver.py:276-281
                my_oper += du;
                if (du > (double)((cap >> 2) * 3)) sp.overflow = 1;  // its row alone outgrows the table
            }
            if (my_oper != 0.0) atomicAdd(&sp.oper, my_oper);
            if (threadIdx.x == 0) {
                sp.nxt_cnt = 0;
                sp.nlong = 0;
                sp.rounds += 1;
                sp.col_nodes += (unsigned long long)nf;
            }
            __syncthreads();
            // ---- SCATTER: a warp per frontier row, an edge per lane; rows of
            // kSpLong edges or more (up to kSpLongMax a round) by the whole block ----
            for (int i = warp; i < nf; i += kWarps) {
                const int u = __ldcg(&keys[cur[i]]);
                const int len = g.row_len[u];
                if (len >= kSpLong) {
                    int slot = kSpLongMax;
                    if (lane == 0) slot = atomicAdd(&sp.nlong, 1);
                    slot = __shfl_sync(kFull, slot, 0);
                    if (slot < kSpLongMax) {
                        if (lane == 0) sp.long_idx[slot] = i;
                        continue;
                    }
                }
                const int64_t rp = g.row_ptr[u];
                const double pv = push[i];
                for (int j0 = 0; j0 < len; j0 += 32)
                    sp_push_edge(g, sp, keys, used_list, R, nxt, cap, theta, j0 + lane < len, rp + j0 + lane, pv);
            }
            __syncthreads();
            const int nlong = min(sp.nlong, kSpLongMax);
            for (int k = 0; k < nlong; ++k) {
                const int i = sp.long_idx[k];
                const int u = __ldcg(&keys[cur[i]]);
                const int64_t rp = g.row_ptr[u];
                const int len = g.row_len[u];
                const double pv = push[i];
                for (int j0 = 0; j0 < len; j0 += kThreads)
                    sp_push_edge(g, sp, keys, used_list, R, nxt, cap, theta, j0 + (int)threadIdx.x < len,
                                 rp + j0 + threadIdx.x, pv);
            }
            __syncthreads();
            if (sp.overflow) break;
            const int nn = sp.nxt_cnt;
            __syncthreads();
            if (threadIdx.x == 0) sp.cur_cnt = nn;
            par ^= 1;
            __syncthreads();
        }
        // ---- result into the query's {x, c} slab, or back to the dense slots ----
        const bool ovf = sp.overflow != 0;
        const int lim = (cap >> 2) * 3;
        const int nu = min(sp.used, lim);
        if (!ovf) {
            float2* xs = reinterpret_cast<float2*>(reinterpret_cast<float*>(a.X) + (int64_t)qid * a.xtile);
            for (int i = threadIdx.x; i < nu; i += kThreads) {
                const int h = used_list[i];
                const double x = X[h];
                const float hi = (float)x;
                xs[__ldcg(&keys[h])] = make_float2(hi, (float)((double)hi - x));  // read out as x - c
            }
        }
        // clear the entries this query used: the table starts empty for the next
        if (sp.used > lim) {
            // a full table holds entries that never reached the used list
            for (int h = threadIdx.x; h < cap; h += kThreads) {
                keys[h] = kSpEmpty;
                R[h] = 0.0;
                X[h] = 0.0;
            }
        } else {
            for (int i = threadIdx.x; i < nu; i += kThreads) {
                const int h = used_list[i];
                keys[h] = kSpEmpty;
                R[h] = 0.0;
                X[h] = 0.0;
            }
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            if (ovf) {
                const int pos = atomicAdd(q.ovf_cnt, 1);
                *(volatile int*)&q.ovf[pos] = qid;
                atomicAdd(&a.stats->sp_ovf, 1ull);
            } else {
                atomicAdd(&a.stats->sp_done, 1ull);
                q.oper[qid] = sp.oper;
                q.rounds[qid] = sp.rounds;
                q.finish_ns[qid] = globaltimer_ns();
                acc_nodes += sp.col_nodes;
                acc_vol += sp.oper;
            }
            __threadfence();
            atomicSub(q.sp_left, 1);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && acc_nodes) {
        atomicAdd(&a.stats->col_nodes, acc_nodes);
        atomicAdd(&a.stats->union_nodes, acc_nodes);
        atomicAdd(&a.stats->col_vol, acc_vol);
        atomicAdd(&a.stats->union_vol, acc_vol);
    }
}

// Opt-in per-block phase timeline (thread 0, first trace_iters iterations).
__device__ __forceinline__ void trace_point(const PushArgs& a, int it, int k) {
    if (a.trace && it < a.trace_iters && threadIdx.x == 0)
        a.trace[((size_t)it * gridDim.x + blockIdx.x) * kTracePoints + k] = globaltimer_ns();
}

template <typename T, int W>
__global__ void __launch_bounds__(kThreads, (W == 1 && sizeof(T) == 4)   ? GDE_MIN_BLOCKS_W1
                                           : (W <= 8 && sizeof(T) == 4) ? GDE_MIN_BLOCKS_F32
                                                                        : GDE_MIN_BLOCKS)
    push_kernel(PushArgs a) {
    __shared__ TileSh sh;
    __shared__ PrepSh ps;
    __shared__ RoundSh rs;
    __shared__ int s_cnt[kMaxW];
    __shared__ long long s_vals[kMaxLaunchTiles];
    const int64_t n = a.g.n;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.stats->start_ns = globaltimer_ns();
    if (threadIdx.x == 0) {
        ps.acc_col_nodes = 0; ps.acc_union_nodes = 0;
        ps.acc_col_vol = 0.0; ps.acc_union_vol = 0.0;
    }
    // the launch's last sp_blocks blocks solve small queries out of hash tables
    if (a.serve && a.queue.sp_blocks > 0 && (int)blockIdx.x >= (int)gridDim.x - a.queue.sp_blocks) {
        sparse_block_loop(a, (int)blockIdx.x - ((int)gridDim.x - a.queue.sp_blocks));
        return;
    }
    int it = 0;
    const bool online = a.serve && a.queue.online;
    const GroupInfo gi = group_of(a);
    const int G = a.groups > 1 ? a.groups : 1;
    if (online && blockIdx.x == 0 && threadIdx.x == 0) *a.queue.last_ns = globaltimer_ns();
    for (; it < a.round_budget; ++it) {
        // online server: group 0 decided to stop (stop flag, or idle), and this
        // group took its copy of the decision before last round's barrier
        if (online && ld_volatile_i(a.queue.gquit + gi.id) != 0) break;
        trace_point(a, it, TP_ITER);
        // ---- live tiles of this round (identical in every block) ----
        if (threadIdx.x == 0) { rs.any_check = 0; rs.any_idle = 0; rs.ndrain = 0; }
        __syncthreads();
        for (int t = threadIdx.x; t < a.ntiles; t += kThreads) {
            const TileState& ts = a.ts[t];
            const bool mine = (t % G) == gi.id;  // this group's slots
            const bool live = mine && ts.done == SLOT_LIVE && it >= ts.t0 && (it - ts.t0) < a.max_rounds;
            s_vals[t] = live ? 1 : 0;
            rs.idle[t] = !mine ? 0 : (ts.done == SLOT_IDLE) ? 1 : (ts.done == SLOT_DRAIN ? 2 : 0);
            if (mine && ts.done == SLOT_IDLE) rs.any_idle = 1;
        }
        if (online) {
            // drained slots in ascending order: the same list in every block
            __syncthreads();
            if (threadIdx.x == 0) {
                int nd = 0;
                for (int t = 0; t < a.ntiles; ++t)
                    if (rs.idle[t] == 2) rs.drain[nd++] = (short)t;
                rs.ndrain = nd;
            }
        }
        __syncthreads();
        block_exclusive_scan(s_vals, a.ntiles, rs.off[0], rs.scan_tmp);
        for (int t = threadIdx.x; t < a.ntiles; t += kThreads) {
            if (rs.off[0][t + 1] != rs.off[0][t]) {
                const int k = (int)rs.off[0][t];
                rs.tiles[k] = t;
                rs.level[k] = it - a.ts[t].t0;
                const int m = a.tp[t].method;
                if (m == M_GLOBAL_GD || m == M_GLOBAL_CHEBY || (m == M_HK_GLOBAL && hk_relaxed(a.tp[t])))
                    rs.any_check = 1;
            }
        }
        if (threadIdx.x == 0) rs.ntl = (int)rs.off[0][a.ntiles];
        __syncthreads();
        const int ntl = rs.ntl;
        if (ntl == 0 && !rs.any_idle && rs.ndrain == 0) break;
        const bool timer = (blockIdx.x == 0 && threadIdx.x == 0);
        unsigned long long t0 = timer ? globaltimer_ns() : 0ull;
        // ---- CHECK (global GD / Chebyshev tiles) ----
        if (rs.any_check) {
            for (int k = 0; k < ntl; ++k) {
                const int t = rs.tiles[k];
                const int m = a.tp[t].method;
                if constexpr (sizeof(T) == 8)
                    if (m == M_HK_GLOBAL && hk_relaxed(a.tp[t])) hk_sweeps_phase<T, W>(a, t, it);
                if (m != M_GLOBAL_GD && m != M_GLOBAL_CHEBY) continue;
                check_phase<T, W>(a, t, it, s_cnt);
            }
            if (!grid_barrier(a.bar + gi.id, a.err, a.spin_limit, gi.dim)) return;
            if (timer) {
                unsigned long long t1 = globaltimer_ns();
                a.stats->check_ns += t1 - t0;
                t0 = t1;
            }
        }
        // ---- PREP: flattened candidates of all live tiles ----
        if (gi.blk == 0) {
            for (int k = 0; k < ntl; ++k) zero_next_counters<W>(a, rs.tiles[k], rs.level[k]);
        }
        for (int k = threadIdx.x; k < ntl; k += kThreads) {
            const TileState& ts = a.ts[rs.tiles[k]];
            const int lv = rs.level[k];
            s_vals[k] = ts.dense_next[lv & 1] ? n : ts.cand_cnt[lv % 3];
        }
        __syncthreads();
        block_exclusive_scan(s_vals, ntl, rs.off[0], rs.scan_tmp);
        trace_point(a, it, TP_PREP_WORK);
        {
            long long lo, hi;
            block_share(rs.off[0][ntl], lo, hi, gi);
            if (lo < hi) {
                for (int k = find_tile(rs.off[0], ntl, lo); k < ntl && rs.off[0][k] < hi; ++k) {
                    const long long b = max(lo, rs.off[0][k]) - rs.off[0][k];
                    const long long e = min(hi, rs.off[0][k + 1]) - rs.off[0][k];
                    if (b >= e) continue;
                    load_tile<W>(a, rs.tiles[k], it, sh);
                    prep_range<T, W>(a, rs.tiles[k], sh, ps, b, e);
                }
            }
        }
        trace_point(a, it, TP_PREP_DONE);
        if (!grid_barrier(a.bar + gi.id, a.err, a.spin_limit, gi.dim)) return;
        trace_point(a, it, TP_PREP_BAR);
        if (timer) {
            unsigned long long t1 = globaltimer_ns();
            a.stats->prep_ns += t1 - t0;
            t0 = t1;
        }
        // ---- SCATTER: flattened short rows / medium rows / long-row chunks ----
        for (int k = threadIdx.x; k < ntl; k += kThreads) {
            const int t = rs.tiles[k];
            const TileState& ts = a.ts[t];
            const TileParams& tp = a.tp[t];
            const int lv = rs.level[k];
            const int par = lv & 1;
            const int m = tp.method;
            const bool hk = method_is_hk(m);
            const bool fin = hk && (m != M_HK_TAYLOR) && (lv + 1 == tp.n_levels);
            const bool last_taylor = (m == M_HK_TAYLOR) && (lv >= tp.n_levels);
            const bool dnext = dense_next_round(a, tp, ts, par);
            unsigned char f = 0;
            if (hk) f |= SF_HK;
            if (fin) f |= SF_FINAL;
            if (last_taylor) f |= SF_NOPUSH;
            if (tp.kind == KIND_IGN) f |= SF_TGTSCALE;
            if (tile_crosses(tp)) f |= SF_CROSS;
            else if (!dnext && !fin && !last_taylor) f |= SF_TRACK;
            rs.flags[k] = f;
            const bool has = ts.front_cnt[par] > 0 && !last_taylor;
            s_vals[k] = has ? ts.small_cnt[par] : 0;
        }
        __syncthreads();
        block_exclusive_scan(s_vals, ntl, rs.off[0], rs.scan_tmp);
        for (int k = threadIdx.x; k < ntl; k += kThreads) {
            const TileState& ts = a.ts[rs.tiles[k]];
            const int par = rs.level[k] & 1;
            s_vals[k] = (ts.front_cnt[par] > 0 && !(rs.flags[k] & SF_NOPUSH)) ? ts.med_cnt[par] : 0;
        }
        __syncthreads();
        block_exclusive_scan(s_vals, ntl, rs.off[1], rs.scan_tmp);
        for (int k = threadIdx.x; k < ntl; k += kThreads) {
            const TileState& ts = a.ts[rs.tiles[k]];
            const int par = rs.level[k] & 1;
            s_vals[k] = (ts.front_cnt[par] > 0 && !(rs.flags[k] & SF_NOPUSH)) ? ts.large_cnt[par] : 0;
        }
        __syncthreads();
        block_exclusive_scan(s_vals, ntl, rs.off[2], rs.scan_tmp);
        if (a.serve) {
            // slots whose query finished this round: extract + clear, every
            // block an equal share of the retiring slots' nodes
            for (int k = threadIdx.x; k < ntl; k += kThreads) {
                const TileState& ts = a.ts[rs.tiles[k]];
                s_vals[k] = (ts.front_cnt[rs.level[k] & 1] == 0) ? n : 0;
            }
            __syncthreads();
            block_exclusive_scan(s_vals, ntl, rs.off[3], rs.scan_tmp);
            long long lo, hi;
            block_share(rs.off[3][ntl], lo, hi, gi);
            if (lo < hi) {
                for (int k = find_tile(rs.off[3], ntl, lo); k < ntl && rs.off[3][k] < hi; ++k) {
                    const long long b = max(lo, rs.off[3][k]) - rs.off[3][k];
                    const long long e = min(hi, rs.off[3][k + 1]) - rs.off[3][k];
                    if (b >= e) continue;
                    if (online) gather_online_range<T, W>(a, rs.tiles[k], b, e);
                    else retire_range<T, W>(a, rs.tiles[k], b, e);
                }
            }
            // online slots drained last round: every block of the group an equal share of their nodes
            if (online && rs.ndrain > 0) {
                block_share((long long)rs.ndrain * n, lo, hi, gi);
                for (long long x = lo; x < hi;) {
                    const long long k = x / n;
                    const long long e = min(hi, (k + 1) * n);
                    clear_slot_range<T, W>(a, rs.drain[k], x - k * n, e - k * n);
                    x = e;
                }
            }
        }
        trace_point(a, it, TP_SCAT_WORK);
        // long-row chunks first (largest pieces), then medium, then short rows
        for (int sp = 2; sp >= 0; --sp) {
            const long long* off = rs.off[sp];
            long long lo, hi;
            block_share(off[ntl], lo, hi, gi);
            if (lo >= hi) continue;
            for (int k = find_tile(off, ntl, lo); k < ntl && off[k] < hi; ++k) {
                const long long b = max(lo, off[k]) - off[k];
                const long long e = min(hi, off[k + 1]) - off[k];
                if (b >= e) continue;
                const int t = rs.tiles[k];
                const ScatterCtx<T, W> c = scatter_ctx<T, W>(a, t, rs.level[k], rs.flags[k]);
                if constexpr (W == 1) {
                    if (sp == 2) scatter_warp_items_w1<T>(a, a.blarge + (int64_t)t * a.large_cap, 1, c, b, e);
                    else if (sp == 1) scatter_warp_items_w1<T>(a, a.bsmall + (int64_t)t * n + (n - 1), -1, c, b, e);
                    else scatter_flat_w1<T, 32>(a, a.bsmall + (int64_t)t * n, 1, c, b, e);
                } else {
                    if (sp == 2) scatter_warp_items<T, W>(a, a.blarge + (int64_t)t * a.large_cap, 1, c, b, e);
                    else if (sp == 1) scatter_warp_items<T, W>(a, a.bsmall + (int64_t)t * n + (n - 1), -1, c, b, e);
                    else scatter_small_flat<T, W>(a, t, c, b, e);
                }
            }
        }
        trace_point(a, it, TP_SCAT_DONE);
        // HK level drop (touches the current level's slab only)
        for (int k = 0; k < ntl; ++k) {
            if (!(rs.flags[k] & SF_HK)) continue;
            const int t = rs.tiles[k];
            const int lv = rs.level[k];
            const TileState& ts = a.ts[t];
            if (ts.front_cnt[lv & 1] == 0) continue;
            hk_drop<T, W>(a, t, lv, ts.dense_next[lv & 1] != 0, ts.cand_cnt[lv % 3], gi);
        }
        bool admitted = false;
        if (gi.blk == 0 && online) {
            if (threadIdx.x == 0) {
                for (int k = 0; k < rs.ndrain; ++k) {
                    publish_online(a, rs.drain[k]);
                    a.ts[rs.drain[k]].done = SLOT_IDLE;  // admitted from the next round on
                }
                if (gi.id == 0 && route_online(a)) admitted = true;
                if (rs.any_idle)
                    for (int t = 0; t < a.ntiles; ++t)
                        if (rs.idle[t] == 1 && admit_online<T, W>(a, t, it)) admitted = true;
            }
        } else if (gi.blk == 0 && a.serve && rs.any_idle) {
            for (int t = 0; t < a.ntiles; ++t)
                if (rs.idle[t] == 1) admit_query<T, W>(a, t, it);
        }
        if (gi.blk == 0) {
            finish_columns_all<W>(a, rs, ntl);
            __syncthreads();
            for (int k = threadIdx.x; k < ntl; k += kThreads) {
                const int t = rs.tiles[k];
                const int lv = rs.level[k];
                const bool dnext = dense_next_round(a, a.tp[t], a.ts[t], lv & 1);
                finish_round<W>(a, t, lv, dnext);
            }
            if (online && threadIdx.x == 0) {
                // a slot that reaches max_rounds ends with GDE_EITERCAP (its row is not written)
                for (int k = 0; k < ntl; ++k) {
                    const int t = rs.tiles[k];
                    TileState& ts = a.ts[t];
                    if (ts.done == SLOT_LIVE && it + 1 - ts.t0 >= a.max_rounds) {
                        OnlineSlot& os = a.queue.slot[t];
                        os.oper = a.cs[(int64_t)t * W].oper;
                        os.rounds = a.cs[(int64_t)t * W].rounds;
                        os.finish_ns = globaltimer_ns();
                        os.status = GDE_EITERCAP;
                        ts.done = SLOT_DRAIN;
                    }
                }
                // Group 0 decides for the server: leave on the stop flag, or
                // after idle_ns with nothing live, draining, in a mailbox or in
                // the ring in any group (every slot is then idle: a later
                // launch picks the ring up where this one left it).  Every
                // group takes its copy of the decision before its barrier.
                if (gi.id == 0) {
                    const unsigned long long now = globaltimer_ns();
                    bool busy = ntl > 0 || rs.ndrain > 0 || admitted || *a.queue.head < ld_acquire_sys(a.queue.tail);
                    for (int t = 0; t < a.ntiles && !busy; ++t)
                        busy = ld_volatile_i(&a.queue.slot[t].pending) != 0 || ld_volatile_i(&a.ts[t].done) != SLOT_IDLE;
                    if (busy) *a.queue.last_ns = now;
                    if (ld_relaxed_sys_i(a.queue.stop) != 0 || (!busy && now - *a.queue.last_ns > a.queue.idle_ns))
                        *(volatile int*)a.queue.quit = 1;
                }
                a.queue.gquit[gi.id] = ld_volatile_i(a.queue.quit);
            }
        }
        trace_point(a, it, TP_SCAT_ENTER);
        if (!grid_barrier(a.bar + gi.id, a.err, a.spin_limit, gi.dim)) return;
        trace_point(a, it, TP_SCAT_BAR);
        if (timer) a.stats->scatter_ns += globaltimer_ns() - t0;
    }
    // A tile still SLOT_LIVE after the launch stopped at max_rounds (the host
    // reports GDE_EITERCAP for it).
    if (gi.blk == 0 && threadIdx.x == 0) atomicMax(&a.stats->iters, (unsigned long long)it);
    if (threadIdx.x == 0 && ps.acc_union_nodes) {
        atomicAdd(&a.stats->col_nodes, ps.acc_col_nodes);
        atomicAdd(&a.stats->col_vol, ps.acc_col_vol);
        atomicAdd(&a.stats->union_nodes, ps.acc_union_nodes);
        atomicAdd(&a.stats->union_vol, ps.acc_union_vol);
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
