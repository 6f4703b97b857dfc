// aux_kernels.cu -- column initialisation, result extraction, graph edits.
#include <cuda_runtime.h>

#include <algorithm>

#include "gde_common.cuh"
#include "gde_device.cuh"
#include "gde_engine.h"

namespace gde {

namespace {

// One warp per column: set the seed's residual (and the Chebyshev start
// x1 = a e_s, r1 = (1-a) A D^-1 a e_s, ppr_solver.py:587-601; katz_solver.py:
// 345-355), push `push0` to the seed's neighbours, and append the touched
// nodes to the tile's round-0 candidate list (deduplicated across columns).
template <typename T>
__global__ void init_columns_kernel(PushArgs a, const InitCol* cols, int ncols, int W) {
    int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (wid >= ncols) return;
    InitCol ic = cols[wid];
    const int64_t n = a.g.n;
    const int64_t base = (int64_t)ic.tile * a.tile_stride;
    const int64_t xld = a.xld ? a.xld : a.ld;  // X may interleave {x, Kahan term}
    T* R = reinterpret_cast<T*>(a.R) + base;
    T* X = reinterpret_cast<T*>(a.X) + (int64_t)ic.tile * (a.xld ? a.xtile : a.tile_stride);
    T* DX = a.DX ? reinterpret_cast<T*>(a.DX) + base : nullptr;
    int32_t* mark = a.mark + (int64_t)ic.tile * n;
    int32_t* list = a.cand + ((int64_t)ic.tile * 2 + 0) * n;
    int* cnt = &a.ts[ic.tile].cand_cnt[0];
    const int stamp = a.ts[ic.tile].stamp;
    const int64_t so = (int64_t)ic.seed * a.ld + ic.col;
    if (lane == 0) {
        // served FP32 PPR / Katz local GD slots keep the hub prefix's residual in FP64
        const TileParams& tp = a.tp[ic.tile];
        const bool crosses = tp.method == M_LOCAL_GD && (tp.kind == KIND_PPR || tp.kind == KIND_KATZ);
        if (sizeof(T) == 4 && a.RH && crosses && ic.seed < a.rh_cut)
            a.RH[(int64_t)ic.tile * a.rh_cut + ic.seed] = ic.r0;
        else
            R[so] = (T)ic.r0;
        if (ic.x0 != 0.0) X[(int64_t)ic.seed * xld + ic.col] = (T)ic.x0;
        if (DX && ic.dx0 != 0.0) DX[so] = (T)ic.dx0;
    }
    __syncwarp();
    append_once(lane == 0, ic.seed, mark, stamp, list, cnt, 0xffffffffu);
    if (ic.push0 != 0.0) {
        const int64_t rp = a.g.row_ptr[ic.seed];
        const int len = a.g.row_len[ic.seed];
        for (int j0 = 0; j0 < len; j0 += 32) {
            int j = j0 + lane;
            bool ok = j < len;
            int v = ok ? a.g.col[rp + j] : 0;
            if (ok) atomicAdd(R + (int64_t)v * a.ld + ic.col, (T)ic.push0);
            append_once(ok, v, mark, stamp, list, cnt, 0xffffffffu);
        }
    }
}

template <typename T, typename O>
__global__ void extract_kernel(PushArgs a, const ExtractCol* cols, O* x_out, O* r_out, int64_t ld_out, int64_t n,
                               int clear) {
    const ExtractCol ec = cols[blockIdx.y];
    const int64_t base = (int64_t)ec.tile * a.tile_stride + ec.col;
    const int64_t xbase = (int64_t)ec.tile * (a.xld ? a.xtile : a.tile_stride) + ec.col;
    const int64_t xld = a.xld ? a.xld : a.ld;  // X may interleave {x, Kahan term}
    T* X = reinterpret_cast<T*>(a.X) + xbase;
    T* R = reinterpret_cast<T*>(a.R) + base;
    T* R2 = a.R2 ? reinterpret_cast<T*>(a.R2) + base : nullptr;
    float* XC = a.XC ? a.XC + xbase : nullptr;  // Kahan compensation: the sum is X - XC
    const int rl = ec.r_levels;
    const int32_t* perm = a.g.perm;
    // u runs over caller ids; the slabs are in internal (relabelled) order
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = perm ? (int64_t)perm[u] : u;
        const int64_t o = v * a.ld, xo = v * xld;
        if (x_out) {
            double x = (double)X[xo];
            if (XC) x -= (double)XC[xo];
            if (u == ec.seed) x = x + ec.seed_add;
            if (ec.scale != 1.0) x = x / ec.scale;
            x_out[ec.out_row * ld_out + u] = (O)x;
        }
        if (r_out) {
            r_out[ec.out_row * rl * ld_out + u] = (O)R[o];
            if (rl == 2) r_out[(ec.out_row * rl + 1) * ld_out + u] = R2 ? (O)R2[o] : (O)0;
        }
        if (clear) {
            X[xo] = T(0);
            R[o] = T(0);
            if (R2) R2[o] = T(0);
            if (XC) XC[xo] = 0.f;
        }
    }
}

// dst row u (caller order) <- src row perm[u] (internal order), or the reverse
template <typename T>
__global__ void permute_rows_kernel(const T* src, int64_t sld, T* dst, int64_t dld, const int32_t* perm, int64_t n,
                                    int64_t F, int to_internal) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * F; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t u = i / F, c = i % F;
        const int64_t p = perm[u];
        if (to_internal) dst[p * dld + c] = src[u * sld + c];
        else dst[u * dld + c] = src[p * sld + c];
    }
}

// per row r: dst[r][u] (caller order) <- src[r][perm[u]] (internal order)
template <typename T>
__global__ void permute_entries_kernel(const T* src, int64_t sld, T* dst, int64_t dld, const int32_t* perm, int64_t n,
                                       int64_t rows) {
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y)
        for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x)
            dst[r * dld + u] = src[r * sld + perm[u]];
}

// Served solutions kept per query as interleaved {x, Kahan term} slabs:
// out[q][u] (caller order) = x - c at internal node perm[u], plus the Katz
// seed correction xt[s_node] -= 1 (katz_solver.py:243) and the heat
// kernel's xt / e^tau (hk_solver.py:295).
template <typename O>
__global__ void query_rows_kernel(const float* XI, int64_t xtile, const int32_t* perm, int64_t n, int64_t nq,
                                  const int32_t* seed_int, const int32_t* kinds, double seed_add, double hk_scale,
                                  O* out, int64_t ld_out) {
    // rows by blockIdx.y, nodes by blockIdx.x: no 64-bit division per entry
    for (int64_t q = blockIdx.y; q < nq; q += gridDim.y) {
        const float* xq = XI + q * xtile;
        const int64_t s = seed_int[q];
        const double add = kinds ? (kinds[q] == KIND_KATZ ? -1.0 : 0.0) : seed_add;
        const bool hk = kinds && kinds[q] == KIND_HK;
        O* oq = out + q * ld_out;
        for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
            const int64_t v = perm ? (int64_t)perm[u] : u;
            const float2 xc = *reinterpret_cast<const float2*>(xq + 2 * v);
            double x = (double)xc.x - (double)xc.y;
            if (v == s) x += add;
            if (hk) x = x / hk_scale;
            oq[u] = (O)x;
        }
    }
}

// The same read-out walking each slab in internal order (sequential {x, c}
// reads) and scattering into the caller-order row, which stays in L2 while
// it is written; used for device rows.
template <typename O>
__global__ void query_rows_scatter_kernel(const float* XI, int64_t xtile, const int32_t* iperm, int64_t n, int64_t nq,
                                          const int32_t* seed_int, const int32_t* kinds, double seed_add,
                                          double hk_scale, O* out, int64_t ld_out) {
    for (int64_t q = blockIdx.y; q < nq; q += gridDim.y) {
        const float2* xq = reinterpret_cast<const float2*>(XI + q * xtile);
        const int64_t s = seed_int[q];
        const double add = kinds ? (kinds[q] == KIND_KATZ ? -1.0 : 0.0) : seed_add;
        const bool hk = kinds && kinds[q] == KIND_HK;
        O* oq = out + q * ld_out;
        for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
            const float2 xc = xq[v];
            double x = (double)xc.x - (double)xc.y;
            if (v == s) x += add;
            if (hk) x = x / hk_scale;
            oq[iperm[v]] = (O)x;
        }
    }
}

// Per-node degree tables of the nodes an edge batch touched (rec[i] for node
// ids[i]); the InstantGNN tables only when nf is given.
__global__ void node_tables_kernel(int64_t nn, const NodeTables* rec, int32_t* row_len, double* degd, float* degf,
                                   double* nfac, double* tfac, float* tfac_f) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x) {
        const NodeTables r = rec[i];
        row_len[r.id] = r.len;
        degd[r.id] = r.degd;
        degf[r.id] = (float)r.degd;
        if (nfac) {
            nfac[r.id] = r.nf;
            tfac[r.id] = r.tf;
            tfac_f[r.id] = (float)r.tf;
        }
    }
}

__global__ void apply_entries_kernel(int32_t* col, const int64_t* pos, const int32_t* val, int64_t k) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < k; i += (int64_t)gridDim.x * blockDim.x)
        col[pos[i]] = val[i];
}

}  // namespace

cudaError_t init_columns(const PushArgs& a, int prec64, int W, const InitCol* d_cols, int ncols, cudaStream_t st) {
    if (ncols == 0) return cudaSuccess;
    int blocks = (ncols * 32 + 255) / 256;
    if (prec64) init_columns_kernel<double><<<blocks, 256, 0, st>>>(a, d_cols, ncols, W);
    else init_columns_kernel<float><<<blocks, 256, 0, st>>>(a, d_cols, ncols, W);
    return cudaGetLastError();
}

cudaError_t extract_columns(const PushArgs& a, int prec64, int W, const ExtractCol* d_cols, int ncols, void* x_out,
                            void* r_out, int out64, int64_t ld_out, int64_t n, int clear, cudaStream_t st) {
    if (ncols == 0) return cudaSuccess;
    int bx = (int)((n + 255) / 256);
    if (bx > 1024) bx = 1024;
    dim3 grid(bx, ncols);
    if (prec64) {
        if (out64) extract_kernel<double, double><<<grid, 256, 0, st>>>(a, d_cols, (double*)x_out, (double*)r_out, ld_out, n, clear);
        else extract_kernel<double, float><<<grid, 256, 0, st>>>(a, d_cols, (float*)x_out, (float*)r_out, ld_out, n, clear);
    } else {
        if (out64) extract_kernel<float, double><<<grid, 256, 0, st>>>(a, d_cols, (double*)x_out, (double*)r_out, ld_out, n, clear);
        else extract_kernel<float, float><<<grid, 256, 0, st>>>(a, d_cols, (float*)x_out, (float*)r_out, ld_out, n, clear);
    }
    return cudaGetLastError();
}

cudaError_t permute_rows(const void* src, int64_t sld, void* dst, int64_t dld, const int32_t* perm, int64_t n,
                         int64_t F, int elem, int to_internal, cudaStream_t st) {
    if (n == 0 || F == 0) return cudaSuccess;
    int64_t total = n * F;
    int blocks = (int)std::min<int64_t>((total + 255) / 256, 8192);
    if (elem == 8)
        permute_rows_kernel<double><<<blocks, 256, 0, st>>>((const double*)src, sld, (double*)dst, dld, perm, n, F,
                                                             to_internal);
    else
        permute_rows_kernel<float><<<blocks, 256, 0, st>>>((const float*)src, sld, (float*)dst, dld, perm, n, F,
                                                            to_internal);
    return cudaGetLastError();
}

cudaError_t permute_entries(const void* src, int64_t sld, void* dst, int64_t dld, const int32_t* perm, int64_t n,
                            int64_t rows, int elem, cudaStream_t st) {
    if (n == 0 || rows == 0) return cudaSuccess;
    const dim3 blocks((unsigned)std::min<int64_t>((n + 255) / 256, 2048), (unsigned)std::min<int64_t>(rows, 65535));
    if (elem == 8)
        permute_entries_kernel<double><<<blocks, 256, 0, st>>>((const double*)src, sld, (double*)dst, dld, perm, n,
                                                                rows);
    else
        permute_entries_kernel<float><<<blocks, 256, 0, st>>>((const float*)src, sld, (float*)dst, dld, perm, n, rows);
    return cudaGetLastError();
}

cudaError_t query_rows(const float* XI, int64_t xtile, const int32_t* perm, const int32_t* iperm, int64_t n,
                       int64_t nq, const int32_t* seed_int, const int32_t* kinds, double seed_add, double hk_scale,
                       void* out, int out64, int64_t ld_out, cudaStream_t st) {
    if (n == 0 || nq == 0) return cudaSuccess;
    const dim3 blocks((unsigned)std::min<int64_t>((n + 255) / 256, 2048), (unsigned)std::min<int64_t>(nq, 65535));
    if (iperm) {
        if (out64)
            query_rows_scatter_kernel<double><<<blocks, 256, 0, st>>>(XI, xtile, iperm, n, nq, seed_int, kinds,
                                                                       seed_add, hk_scale, (double*)out, ld_out);
        else
            query_rows_scatter_kernel<float><<<blocks, 256, 0, st>>>(XI, xtile, iperm, n, nq, seed_int, kinds,
                                                                      seed_add, hk_scale, (float*)out, ld_out);
        return cudaGetLastError();
    }
    if (out64)
        query_rows_kernel<double><<<blocks, 256, 0, st>>>(XI, xtile, perm, n, nq, seed_int, kinds, seed_add, hk_scale,
                                                           (double*)out, ld_out);
    else
        query_rows_kernel<float><<<blocks, 256, 0, st>>>(XI, xtile, perm, n, nq, seed_int, kinds, seed_add, hk_scale,
                                                          (float*)out, ld_out);
    return cudaGetLastError();
}

cudaError_t node_tables(int64_t nn, const NodeTables* rec, int32_t* row_len, double* degd, float* degf, double* nfac,
                        double* tfac, float* tfac_f, cudaStream_t st) {
    if (nn == 0) return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((nn + 255) / 256, 4096);
    node_tables_kernel<<<blocks, 256, 0, st>>>(nn, rec, row_len, degd, degf, nfac, tfac, tfac_f);
    return cudaGetLastError();
}

cudaError_t graph_apply_entries(int32_t* col, const int64_t* pos, const int32_t* val, int64_t k, cudaStream_t st) {
    if (k == 0) return cudaSuccess;
    int blocks = (int)((k + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    apply_entries_kernel<<<blocks, 256, 0, st>>>(col, pos, val, k);
    return cudaGetLastError();
}

}  // namespace gde
