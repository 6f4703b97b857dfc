// spectral.cu -- extreme eigenvalues of the adjacency matrix on the GPU, for
// the Chebyshev bounds of Katz (katz_cheby takes l_max, mu_min of
// Q = I - alpha A, katz_solver.py:340-368).
//
// The reference obtains lambda_max(A) and lambda_min(A) with
// scipy.sparse.linalg.eigsh (katz_exp_dmax.py:20, katz_exp_dmin.py:20).  Here
// a Lanczos iteration runs on the device -- FP64 adjacency products (one warp
// per row), dot products and vector updates -- and the host finds the
// extreme eigenvalues of the small tridiagonal matrix by Sturm-sequence
// bisection.  Extreme Ritz values converge first and are not disturbed by
// the loss of orthogonality that plain Lanczos suffers in its interior.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "gde_common.cuh"
#include "gde_engine.h"

void gde_internal_set_lam_max(gde_graph* G, double lam);

using namespace gde;

int gde_internal_fail(gde_ctx* ctx, int code, const char* msg);
cudaStream_t gde_internal_stream(gde_ctx* ctx);
int gde_internal_device(gde_ctx* ctx);
const DevGraph* gde_internal_devgraph(gde_graph* G);
void* gde_internal_wsget(gde_ctx* ctx, const char* name, size_t bytes);

namespace {

constexpr int kThreads = 256;
constexpr int kDotBlocks = 1024;

// y = A x (A the graph's unweighted adjacency; row u holds row_len[u] entries)
__global__ void adj_spmv_kernel(DevGraph g, const double* __restrict__ x, double* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = warp; u < g.n; u += nwarps) {
        const int64_t rp = g.row_ptr[u];
        const int len = g.row_len[u];
        double s = 0.0;
        for (int j = lane; j < len; j += 32) s += x[g.col[rp + j]];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) y[u] = s;
    }
}

// partial[b] = sum over block b's share of a[i] * b[i]
__global__ void dot_kernel(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                           double* __restrict__ partial) {
    __shared__ double sh[kThreads / 32];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += a[i] * b[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += sh[w];
        partial[blockIdx.x] = t;
    }
}

// w = w - a * v - b * vp
__global__ void lanczos_update_kernel(double* __restrict__ w, const double* __restrict__ v,
                                      const double* __restrict__ vp, double a, double b, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        w[i] = w[i] - a * v[i] - b * vp[i];
}

// y = x * s
__global__ void scale_kernel(const double* __restrict__ x, double s, double* __restrict__ y, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = x[i] * s;
}

// deterministic start vector: 1 + small hash-based perturbation per node
__global__ void start_vector_kernel(double* v, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        unsigned long long z = (unsigned long long)i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
        z ^= z >> 31;
        z *= 0xBF58476D1CE4E5B9ull;
        z ^= z >> 29;
        v[i] = 1.0 + 0.5 * ((double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5);
    }
}

// Number of eigenvalues of the symmetric tridiagonal (a, b) below x (Sturm count).
int sturm_below(const std::vector<double>& a, const std::vector<double>& b, int k, double x) {
    int cnt = 0;
    double q = 1.0;
    for (int i = 0; i < k; ++i) {
        const double off = (i > 0) ? b[i] * b[i] : 0.0;
        q = a[i] - x - (i > 0 ? off / q : 0.0);
        if (q == 0.0) q = -1e-300;
        if (q < 0.0) ++cnt;
    }
    return cnt;
}

// Largest and smallest eigenvalue of T_k by bisection to relative tolerance.
void tridiag_extremes(const std::vector<double>& a, const std::vector<double>& b, int k, double* lo_out,
                      double* hi_out) {
    double lo = a[0], hi = a[0];
    for (int i = 0; i < k; ++i) {
        const double r = (i > 0 ? std::fabs(b[i]) : 0.0) + (i + 1 < k ? std::fabs(b[i + 1]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
    }
    auto kth = [&](int target) {  // the (target+1)-th smallest eigenvalue
        double l = lo, h = hi;
        for (int it = 0; it < 200 && h - l > 1e-15 * std::max(1.0, std::fabs(l) + std::fabs(h)); ++it) {
            const double m = 0.5 * (l + h);
            if (sturm_below(a, b, k, m) > target) h = m;
            else l = m;
        }
        return 0.5 * (l + h);
    };
    *lo_out = kth(0);
    *hi_out = kth(k - 1);
}

}  // namespace

extern "C" int gde_katz_spectral_bounds(gde_ctx* ctx, gde_graph* G, double alpha, int max_iter, double tol,
                                        double* lam_max, double* lam_min, double* l_max, double* mu_min) {
    if (!ctx || !G || max_iter < 2) return gde_internal_fail(ctx, GDE_EINVAL, "bad spectral-bound arguments");
    if (!(tol > 0.0)) tol = 1e-10;
    const DevGraph& g = *gde_internal_devgraph(G);
    const int64_t n = g.n;
    cudaStream_t st = gde_internal_stream(ctx);
    if (cudaSetDevice(gde_internal_device(ctx)) != cudaSuccess)
        return gde_internal_fail(ctx, GDE_ECUDA, "cudaSetDevice");
    double* vp = (double*)gde_internal_wsget(ctx, "lz_vp", n * 8);
    double* v = (double*)gde_internal_wsget(ctx, "lz_v", n * 8);
    double* w = (double*)gde_internal_wsget(ctx, "lz_w", n * 8);
    double* part = (double*)gde_internal_wsget(ctx, "lz_part", kDotBlocks * 8);
    if (!vp || !v || !w || !part) return gde_internal_fail(ctx, GDE_ENOMEM, "Lanczos vectors");
    const int blocks = (int)std::min<int64_t>(4096, (n + kThreads - 1) / kThreads);
    std::vector<double> hp(kDotBlocks);
    auto dot = [&](const double* x, const double* y, double* out) -> cudaError_t {
        dot_kernel<<<kDotBlocks, kThreads, 0, st>>>(x, y, n, part);
        cudaError_t e = cudaMemcpyAsync(hp.data(), part, kDotBlocks * 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        double s = 0.0;
        for (double x2 : hp) s += x2;
        *out = s;
        return e;
    };
#define SP_CK(call)                                                                      \
    do {                                                                                 \
        cudaError_t e__ = (call);                                                        \
        if (e__ != cudaSuccess) {                                                        \
            std::string m__ = std::string(#call) + ": " + cudaGetErrorString(e__);      \
            return gde_internal_fail(ctx, GDE_ECUDA, m__.c_str());                       \
        }                                                                                \
    } while (0)
    start_vector_kernel<<<blocks, kThreads, 0, st>>>(w, n);
    SP_CK(cudaGetLastError());
    double nrm2 = 0.0;
    SP_CK(dot(w, w, &nrm2));
    scale_kernel<<<blocks, kThreads, 0, st>>>(w, 1.0 / std::sqrt(nrm2), v, n);
    SP_CK(cudaMemsetAsync(vp, 0, n * 8, st));
    std::vector<double> a, b(1, 0.0);
    double prev_lo = 0.0, prev_hi = 0.0, lo = 0.0, hi = 0.0;
    bool converged = false;
    for (int j = 0; j < max_iter; ++j) {
        adj_spmv_kernel<<<blocks, kThreads, 0, st>>>(g, v, w);
        SP_CK(cudaGetLastError());
        double aj = 0.0;
        SP_CK(dot(w, v, &aj));
        a.push_back(aj);
        lanczos_update_kernel<<<blocks, kThreads, 0, st>>>(w, v, vp, aj, b[j], n);
        double bb = 0.0;
        SP_CK(dot(w, w, &bb));
        const double bj = std::sqrt(std::max(bb, 0.0));
        const int k = (int)a.size();
        if (k >= 2 && (k % 5 == 0 || bj < 1e-12)) {
            tridiag_extremes(a, b, k, &lo, &hi);
            const double scale = std::max(std::fabs(lo), std::fabs(hi));
            if (k >= 10 && std::fabs(hi - prev_hi) <= tol * scale && std::fabs(lo - prev_lo) <= tol * scale) {
                converged = true;
                break;
            }
            prev_lo = lo;
            prev_hi = hi;
        }
        if (bj < 1e-12) {  // invariant subspace: T_k holds exact eigenvalues
            tridiag_extremes(a, b, k, &lo, &hi);
            converged = true;
            break;
        }
        b.push_back(bj);
        // rotate: vp <- v, v <- w / bj
        std::swap(vp, v);
        scale_kernel<<<blocks, kThreads, 0, st>>>(w, 1.0 / bj, v, n);
    }
#undef SP_CK
    if (!converged) tridiag_extremes(a, b, (int)a.size(), &lo, &hi);
    if (converged) gde_internal_set_lam_max(G, hi);  // lets Katz solves judge their distance to the radius
    if (lam_max) *lam_max = hi;
    if (lam_min) *lam_min = lo;
    // eigenvalues of Q = I - alpha A lie in [1 - alpha lam_max, 1 - alpha lam_min]
    if (l_max) *l_max = 1.0 - alpha * lo;
    if (mu_min) *mu_min = 1.0 - alpha * hi;
    return converged ? GDE_OK : gde_internal_fail(ctx, GDE_EITERCAP, "Lanczos did not converge within max_iter");
}
