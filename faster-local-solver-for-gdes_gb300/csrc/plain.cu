// plain.cu -- the plain single-query GPU baseline.
//
// A restatement, on the GB300, of the structure of the reference's CuPy path
// ppr_gd_local_gpu (ppr_solver.py:82-146): one thread per frontier row with a
// serial loop over its edges and an atomicAdd per edge (the kernel string at
// :87-100), dense O(n) passes per round (tmp_rt[:] = 0, rt[:] += tmp_rt,
// nonzero(eps_vec <= |rt|)), FP32 values and thresholds, and one host
// synchronisation per round to learn the frontier size.  The graph stays
// resident (no per-call upload).  This is the denominator of the batched /
// served speed-up, not a product path.
#include <cuda_runtime.h>

#include "gde_common.cuh"
#include "gde_engine.h"

namespace gde {

namespace {

constexpr int kT = 256;

// csr_mat_sparse_vec: thread per frontier row, serial edge loop, atomicAdd
__global__ void plain_csr_kernel(const int32_t* col, const int64_t* row_ptr, const int32_t* row_len, const float* b,
                                 const int32_t* bidx, int nnz_b, float* result) {
    int i = blockDim.x * blockIdx.x + threadIdx.x;
    if (i < nnz_b) {
        int r = bidx[i];
        float v = b[i];
        int64_t e = row_ptr[r] + row_len[r];
        for (int64_t j = row_ptr[r]; j < e; j++) atomicAdd(&result[col[j]], v);
    }
}

// oper += sum(degree[queue[:rear]])
__global__ void plain_oper_kernel(const float* deg, const int32_t* q, int rear, double* oper) {
    __shared__ float s[kT];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    s[threadIdx.x] = (i < rear) ? deg[q[i]] : 0.f;
    __syncthreads();
    for (int o = kT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(oper, (double)s[0]);
}

// sp_vec_data = (1 - alpha) * rt[queue] / degree[queue]
__global__ void plain_sp_kernel(const float* rt, const float* deg, const int32_t* q, int rear, float coef, float* sp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rear) sp[i] = coef * rt[q[i]] / deg[q[i]];
}

// xt[queue] += rt[queue]
__global__ void plain_x_kernel(float* xt, const float* rt, const int32_t* q, int rear) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rear) xt[q[i]] += rt[q[i]];
}

// rt[queue] = 0
__global__ void plain_zero_kernel(float* rt, const int32_t* q, int rear) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < rear) rt[q[i]] = 0.f;
}

// rt[:] += tmp_rt
__global__ void plain_add_kernel(float* rt, const float* tmp, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) rt[i] += tmp[i];
}

// nonzero(eps_vec <= |rt|): per-block counts, scan, ordered write
__global__ void plain_count_kernel(const float* rt, const float* eps_vec, int64_t n, int* bcnt) {
    __shared__ int s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool f = i < n && eps_vec[i] <= fabsf(rt[i]);
    unsigned b = __ballot_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(&s, __popc(b));
    __syncthreads();
    if (threadIdx.x == 0) bcnt[blockIdx.x] = s;
}

__global__ void plain_scan_kernel(int* bcnt, int nb, int* total) {
    // single block exclusive scan over the block counts
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += kT) {
        int i = base + threadIdx.x;
        int v = (i < nb) ? bcnt[i] : 0;
        __shared__ int s[kT];
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kT; o <<= 1) {
            int y = (threadIdx.x >= o) ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += y;
            __syncthreads();
        }
        if (i < nb) bcnt[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == kT - 1) carry += s[kT - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void plain_write_kernel(const float* rt, const float* eps_vec, int64_t n, const int* boff, int32_t* q) {
    __shared__ int wbase[kT / 32];
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool f = i < n && eps_vec[i] <= fabsf(rt[i]);
    unsigned b = __ballot_sync(0xffffffffu, f);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) wbase[w] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int k = 0; k < kT / 32; ++k) { int c = wbase[k]; wbase[k] = acc; acc += c; }
    }
    __syncthreads();
    if (f) q[boff[blockIdx.x] + wbase[w] + __popc(b & ((1u << lane) - 1u))] = (int32_t)i;
}

__global__ void plain_init_kernel(float* xt, float* rt, float* eps_vec, const float* deg, int64_t n, float eps_alpha,
                                  int seed, float alpha, int32_t* q) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        xt[i] = 0.f;
        rt[i] = (i == seed) ? alpha : 0.f;
        eps_vec[i] = eps_alpha * deg[i];
    }
    if (i == 0) q[0] = seed;
}

}  // namespace

int plain_ppr_local(const DevGraph& g, PlainWork& w, int seed, double alpha, double eps, double* oper, int* rounds,
                    cudaStream_t st) {
    const int64_t n = g.n;
    const int nb = (int)((n + kT - 1) / kT);
    plain_init_kernel<<<nb, kT, 0, st>>>(w.xt, w.rt, w.eps_vec, w.degf, n, (float)(eps * alpha), seed, (float)alpha,
                                         w.queue);
    cudaMemsetAsync(w.d_oper, 0, sizeof(double), st);
    int rear = 1;
    int r = 0;
    const float coef = (float)(1.0 - alpha);
    for (;;) {
        if (rear > 0) plain_oper_kernel<<<(rear + kT - 1) / kT, kT, 0, st>>>(w.degf, w.queue, rear, w.d_oper);
        if (rear == 0) break;
        const int qb = (rear + kT - 1) / kT;
        plain_sp_kernel<<<qb, kT, 0, st>>>(w.rt, w.degf, w.queue, rear, coef, w.sp);
        plain_x_kernel<<<qb, kT, 0, st>>>(w.xt, w.rt, w.queue, rear);
        plain_zero_kernel<<<qb, kT, 0, st>>>(w.rt, w.queue, rear);
        cudaMemsetAsync(w.tmp, 0, n * sizeof(float), st);
        plain_csr_kernel<<<(rear + 1023) / 1024, 1024, 0, st>>>(g.col, g.row_ptr, g.row_len, w.sp, w.queue, rear,
                                                                  w.tmp);
        plain_add_kernel<<<nb, kT, 0, st>>>(w.rt, w.tmp, n);
        plain_count_kernel<<<nb, kT, 0, st>>>(w.rt, w.eps_vec, n, w.nz);
        plain_scan_kernel<<<1, kT, 0, st>>>(w.nz, nb, w.d_count);
        plain_write_kernel<<<nb, kT, 0, st>>>(w.rt, w.eps_vec, n, w.nz, w.queue);
        cudaMemcpyAsync(w.h_count, w.d_count, sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);  // rear = len(non_zeros)
        if (e != cudaSuccess) return GDE_ECUDA;
        rear = *w.h_count;
        ++r;
        if (r > 100000) return GDE_EITERCAP;
    }
    cudaMemcpyAsync(oper, w.d_oper, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return GDE_ECUDA;
    *rounds = r;
    return GDE_OK;
}

}  // namespace gde
