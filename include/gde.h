/*
 * gde.h -- C ABI of the GB300 local push solvers for graph diffusion equations.
 *
 * Plain C types only (pointers, sizes, doubles); no CUDA or PyTorch types.
 * Every entry point returns a gde_status (0 = GDE_OK); gde_last_error()
 * gives the message of the last failure on a context.  Pointers marked
 * "host" are ordinary CPU memory; pointers marked "device" are CUDA device
 * memory on the context's device.  Calls on one context are serialised on
 * the context's CUDA stream; distinct contexts may be used from distinct
 * threads.
 *
 * The reference exposes these operations as Python functions
 * (ppr_solver.py, katz_solver.py, hk_solver.py, InstantGNN.py); each entry
 * point below names the functions it replaces.  The drop-in Python modules
 * bind these entry points with ctypes (gde/_lib.py).
 */
#ifndef GDE_H_
#define GDE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference reports failures only by `assert`) ---- */
#define GDE_OK 0
#define GDE_EINVAL 1     /* bad argument (e.g. eps*degree[s] > 1, ppr_solver.py:213) */
#define GDE_ENOMEM 2     /* device memory or the admission budget is exhausted */
#define GDE_EITERCAP 3   /* max_rounds reached before the stopping rule held */
#define GDE_ECUDA 4      /* a CUDA call failed */
#define GDE_EHANG 5      /* a bounded device-side wait ran out (kernel returned early) */
#define GDE_ECAPACITY 6  /* a padded CSR row has no slack left for an insertion */
#define GDE_ENOTFOUND 7  /* unknown query id */

/* ---- problem kinds and methods ---- */
#define GDE_PPR 0   /* (I - (1-a) A D^-1) x = a e_s   (ppr_solver.py:18-23) */
#define GDE_KATZ 1  /* (I - a A) x = e_s              (katz_solver.py:177-179) */
#define GDE_HK 2    /* heat kernel Taylor levels      (hk_solver.py:206-295) */
#define GDE_IGN 3   /* InstantGNN feature push        (InstantGNN.py:12-43) */
#define GDE_UPPR 4  /* dynamic PPR update push        (ppr_solver.py:769-821) */

#define GDE_LOCAL_GD 0
#define GDE_GLOBAL_GD 1
#define GDE_LOCAL_CHEBY 2
#define GDE_GLOBAL_CHEBY 3
#define GDE_HK_LOCAL 4
#define GDE_HK_GLOBAL 5
#define GDE_HK_TAYLOR 6

#define GDE_FP64 0
#define GDE_FP32 1  /* FP32 residuals, Kahan-compensated FP32 solution, FP64 threshold tests */

#define GDE_MEM_HOST 0
#define GDE_MEM_DEVICE 1

typedef struct gde_ctx gde_ctx;
typedef struct gde_graph gde_graph;
typedef struct gde_server gde_server;

typedef struct {
    int kind;          /* GDE_PPR / GDE_KATZ / GDE_HK */
    int method;        /* GDE_LOCAL_GD ... GDE_HK_TAYLOR */
    int prec;          /* GDE_FP64 / GDE_FP32 (Katz with alpha * lambda_max >= 0.9 computes in FP64) */
    int tile_w;        /* columns per tile (1,2,4,8,16,32); 0 = autotuned choice */
    double alpha;      /* PPR / Katz alpha */
    double tau;        /* heat-kernel temperature */
    double l_max;      /* Katz Chebyshev spectral bounds (katz_solver.py:341) */
    double mu_min;
    double beta;       /* InstantGNN exponent */
    double omega;      /* relaxation of gde_sor and of the feature push / update (0 or 1 = synchronous push) */
    int max_rounds;    /* 0 = default (100000) */
    int small_max;     /* degree buckets: <= small_max lane group per row, 0 = default */
    int med_max;       /* <= med_max warp per row, else CTA chunks; 0 = default */
    int chunk;         /* edges per CTA chunk; 0 = default */
    int dense_div;     /* next round scans all nodes when vol(frontier) > n/dense_div; 0 = default */
    int slots;         /* served PPR/Katz local GD: concurrent queries (one residual vector each); 0 = default */
    int groups;        /* served: the grid splits into this many block groups, each advancing its own slots
                          (t % groups) behind its own barrier; 0 = default (one group per slot) */
    int sparse_blocks; /* served FP32 PPR / Katz local GD with solution rows: this many blocks of the launch
                          each solve one small query at a time out of an open-addressing table of node
                          entries instead of dense vectors; 0 = off */
    int sparse_cap;    /* entries per table (rounded up to a power of two); 0 = default (65536).  A query
                          that touches more than 3/4 of it moves to the dense slots */
    double sparse_eps; /* queries with eps >= sparse_eps are small (the table class) */
} gde_params;

typedef struct {
    double kernel_ms;           /* device time of the push launches */
    double total_ms;            /* device time of the whole call */
    int64_t rounds;             /* sum over tiles of rounds run */
    int64_t dense_rounds;
    double union_vol;           /* sum_t vol(union frontier)   -> col_idx bytes */
    double col_vol;             /* sum_t sum_c vol(S_t^c)      -> residual update bytes */
    uint64_t union_nodes;       /* sum_t |union frontier| */
    uint64_t col_nodes;         /* sum_t sum_c |S_t^c| */
    int tiles;
    int tile_w;
    double check_ms;            /* push-kernel time split by phase (global-check / prep / scatter), */
    double prep_ms;             /* each including the wait at the phase's closing grid barrier */
    double scatter_ms;
    int edit_path;              /* gde_feature_update: how the edge batch was applied (GDE_EDIT_*) */
    double edit_ms;             /* gde_feature_update: host time from the call to the push (edit + repair) */
    int prec;                   /* gde_solve / gde_serve: the precision computed in (GDE_FP32 / GDE_FP64);
                                   Katz near its convergence radius is promoted to FP64 */
    int64_t sparse_queries;     /* served: queries solved out of hash tables (gde_params.sparse_blocks) */
    int64_t sparse_overflows;   /* served: small queries that outgrew their table and ran in a dense slot */
} gde_stats;

/* gde_stats.edit_path */
#define GDE_EDIT_HOST 0             /* not reported by this library (every batch runs on the device); kept so
                                       the values of the other two stay fixed */
#define GDE_EDIT_DEVICE_INSERT 1    /* insert-only batch on the device, every edge decided in parallel */
#define GDE_EDIT_DEVICE_DATAFLOW 2  /* batch with deletions or self-loops, or an insert-only batch that found a
                                       row full: on the device, as a dataflow over the edges */

/* ---- context / errors ---- */
const char *gde_status_str(int status);
int gde_version(void);
int gde_ctx_create(int device, gde_ctx **out);
int gde_ctx_destroy(gde_ctx *ctx);
const char *gde_last_error(gde_ctx *ctx);
int gde_ctx_sync(gde_ctx *ctx);

/* ---- push-kernel phase trace (diagnostics; no counterpart in the reference) ----
 * gde_ctx_trace(ctx, iters) turns tracing on for the first `iters` launch
 * iterations of every later push launch on this context (0 turns it off).
 * Each block's thread 0 then records %globaltimer (ns) at 8 phase
 * boundaries per iteration: iteration start, PREP work start, PREP work
 * done, PREP barrier passed, SCATTER work start, SCATTER work done,
 * SCATTER barrier entered, SCATTER barrier passed.  gde_ctx_trace_read
 * copies the last launch's stamps to host `out` as
 * out[(iter * grid + block) * points + point] (0 = not reached) and returns
 * the shape; call it with out == NULL to get the shape only. */
int gde_ctx_trace(gde_ctx *ctx, int iters);
int gde_ctx_trace_read(gde_ctx *ctx, uint64_t *out, int64_t cap, int *iters, int *grid, int *points);

/* ---- bounded device waits (failure detection; no counterpart in the reference) ----
 * Every device-side wait of the library is bounded: the push kernel's grid
 * barrier and the edit dataflow's predecessor waits give up after a number of
 * polls, record GDE_EHANG and return, so a wait that cannot end leaves a
 * usable context and an error status instead of a hung GPU.  The defaults are
 * seconds of polling.  gde_ctx_set_wait_limit(ctx, polls) sets the limit of
 * every later wait on this context (0 restores the defaults); a limit of one
 * or two polls makes the waits run out, which is how the GDE_EHANG paths are
 * tested. */
int gde_ctx_set_wait_limit(gde_ctx *ctx, int64_t polls);

/* ---- graph ----
 * Uploads a CSR graph.  Row u's neighbours are indices[indptr[u] ..
 * indptr[u]+row_len[u]); row_len == NULL means indptr[u+1]-indptr[u] (the
 * static layout of ppr_solver.py / katz_solver.py / hk_solver.py); a padded
 * InstantGNN CSR passes its degree array (data_process_GNN.py:93-119).
 * degree == NULL uses the row length as the arithmetic degree (the
 * reference's adj.sum(1), demo.py:44).  `cap` is the length of indices.
 * Replaces the per-call cp.asarray upload of ppr_gd_local_gpu
 * (ppr_solver.py:103-105) with a resident graph. */
int gde_graph_upload(gde_ctx *ctx, int64_t n, int64_t cap, const int64_t *indptr, const int32_t *indices,
                     const int64_t *row_len, const double *degree, gde_graph **out);
int gde_graph_free(gde_graph *g);
int gde_graph_info(gde_graph *g, int64_t *n, int64_t *cap, double *volume);

/* ---- batched single-seed solves ----
 * Solves nq queries (seed[q], eps[q]) of one kind/method in node x column
 * tiles.  Replaces, per query:
 *   ppr_gd(local=True/False)           ppr_solver.py:208-328  (GDE_PPR, LOCAL_GD/GLOBAL_GD, FP64)
 *   ppr_gd_local_gpu / _standard_gpu   ppr_solver.py:82-146, :26-79 (FP32)
 *   ppr_cheby(local=True/False)        ppr_solver.py:582-661  (LOCAL_CHEBY/GLOBAL_CHEBY)
 *   katz_gd, katz_gd_*_gpu             katz_solver.py:167-248, :24-146
 *   katz_cheby                         katz_solver.py:340-431
 *   hk_sor_queue(omega=1)              hk_solver.py:206-295   (HK_LOCAL/HK_GLOBAL)
 *   hk_taylor_approx                   hk_solver.py:51-80     (HK_TAYLOR)
 * x_out / r_out (may be NULL) receive nq rows of ld_out values each (HK
 * r_out: 2 rows per query, the two level buffers of hk_solver.py:212),
 * FP64 when out64 else FP32, in host or device memory per out_mem.
 * seeds / eps are host arrays.  oper_out / rounds_out / lat_ms_out (host,
 * may be NULL) receive the reference's operation count, the rounds, and the
 * device time from the start of the push launch to the round the query
 * finished in. */
int gde_solve(gde_ctx *ctx, gde_graph *g, const gde_params *p, int64_t nq, const int32_t *seeds, const double *eps,
              void *x_out, void *r_out, int out64, int out_mem, int64_t ld_out, double *oper_out,
              int32_t *rounds_out, float *lat_ms_out, gde_stats *stats);

/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or CUDA events with the library's. */
void *gde_ctx_stream(gde_ctx *ctx);

/* ---- served queries (continuous batching) ----
 * PPR / Katz local GD queries served by p->slots concurrent slots inside one
 * persistent launch: a finished query's row is written and its slot handed
 * to the next query on the device.  arrival_ms (host, may be NULL;
 * non-decreasing, queries are admitted in index order): query q is admitted
 * no earlier than arrival_ms[q] after the launch starts, and its latency
 * (lat_ms_out) is measured from that arrival.  gde_solve uses this
 * path for PPR / Katz local GD with tile_w <= 1.  Replaces a loop of
 * ppr_gd_local_gpu / katz_gd_local_gpu calls (ppr_solver.py:82-146,
 * katz_solver.py:81-146) with a request stream. */
int gde_serve(gde_ctx *ctx, gde_graph *g, const gde_params *p, int64_t nq, const int32_t *seeds, const double *eps,
              const double *arrival_ms, void *x_out, void *r_out, int out64, int out_mem, int64_t ld_out,
              double *oper_out, int32_t *rounds_out, float *lat_ms_out, gde_stats *stats);

/* ---- served mixed queries (continuous batching of PPR, Katz and heat kernel) ----
 * kinds[q] in {GDE_PPR, GDE_KATZ, GDE_HK}; alphas[q] the PPR / Katz alpha
 * (host, may be NULL: p->alpha); heat-kernel queries use p->tau and the
 * level push with N = estimate_n(tau, eps/2) (hk_sor_queue, omega = 1,
 * hk_solver.py:206-295).  Each slot takes the kind of the query it admits.
 * hbm_budget_bytes > 0 admits only as many concurrent slots as their
 * vectors fit in that many bytes (GDE_ENOMEM if not even one).  x_out rows
 * are the solutions as the reference returns them (Katz x[s] - 1, heat
 * kernel x / e^tau); arrival_ms and latency as in gde_serve.  Replaces a
 * request loop over ppr_gd_local_gpu / katz_gd_local_gpu / hk_sor_queue
 * calls (ppr_solver.py:82-146, katz_solver.py:81-146, hk_solver.py:206-295). */
int gde_serve_mixed(gde_ctx *ctx, gde_graph *g, const gde_params *p, int64_t nq, const int32_t *kinds,
                    const int32_t *seeds, const double *eps, const double *alphas, const double *arrival_ms,
                    double hbm_budget_bytes, void *x_out, int out64, int out_mem, int64_t ld_out, double *oper_out,
                    int32_t *rounds_out, float *lat_ms_out, gde_stats *stats);

/* ---- online serving: queries submitted while the kernel runs ----
 * Replaces the reference's request loop over single-query solver calls
 * (ppr_solver.py:149-164 over ppr_gd_local_gpu; katz_solver.py:149-164;
 * hk_solver.py:206-295 per seed) with a request stream into one resident
 * persistent launch.  gde_server_start allocates p->slots (default 32, at
 * most 512; fewer if hbm_budget_bytes > 0 holds fewer) one-query slots at
 * precision p->prec, a ring of ring_capacity requests in pinned host memory,
 * and starts a host thread that keeps the push kernel running while there is
 * work: the kernel admits each submitted query into a free slot at a round
 * boundary, advances the live slots in groups that each keep their own round
 * and barrier (p->groups; default one per slot, or one per 8 slots when
 * p->tau >= 1), writes each finished query's
 * solution row (as the reference returns it: Katz x[s] - 1, heat kernel
 * x / e^tau) into the caller's row, and publishes a completion record.
 * After idle_ms with nothing to do the kernel returns; the next submit
 * launches it again.  Heat-kernel queries use the level push with
 * N = estimate_n(p->tau, eps/2) (needs p->tau >= 1); p->tuning fields apply.
 * While the kernel runs it holds every SM; other work on the device waits
 * for it to go idle, and the graph must not be edited.
 *   gde_server_submit: thread-safe, host only; kind GDE_PPR / GDE_KATZ /
 *     GDE_HK, alpha for PPR / Katz; x_out: n entries in caller node order
 *     (FP64 if out64, else FP32), device memory of the context's device or
 *     pinned host memory (or NULL for no row).  *ticket identifies the query.
 *     GDE_ENOMEM when ring_capacity submitted queries are not yet admitted.
 *   gde_server_poll: non-blocking; *done = 1 once the row and the record are
 *     complete, with the operation count, rounds and the device time from
 *     admission to finish.  Records are kept per ticket % ring_capacity: poll
 *     a ticket before ring_capacity later submissions (GDE_ENOTFOUND after).
 *   gde_server_stop: drain != 0 waits for every submitted query first; then
 *     the stop flag ends the kernel at its next round and the server is
 *     freed.  *abandoned (may be NULL) = queries that never finished.
 * Returns GDE_EHANG (through poll or stop) if a bounded device wait ran out. */
int gde_server_start(gde_ctx *ctx, gde_graph *g, const gde_params *p, int64_t ring_capacity,
                     double hbm_budget_bytes, double idle_ms, gde_server **out);
int gde_server_submit(gde_server *s, int kind, int32_t seed, double eps, double alpha, void *x_out, int out64,
                      int64_t *ticket);
int gde_server_poll(gde_server *s, int64_t ticket, int *done, double *oper, int32_t *rounds, double *device_ms);
/* gde_server_poll over k tickets (host arrays; oper, rounds, device_ms may be NULL); returns the first error */
int gde_server_poll_many(gde_server *s, const int64_t *tickets, int64_t k, int32_t *done, double *oper,
                         int32_t *rounds, double *device_ms);
/* slots in use, kernel launches so far, their device time, queries submitted */
int gde_server_info(gde_server *s, int *slots, int64_t *launches, double *kernel_ms, int64_t *submitted);
int gde_server_stop(gde_server *s, int drain, int64_t *abandoned);

/* ---- LocalSOR / APPR (ppr_sor, katz_sor) in multicolour order ----
 * Relaxation res = omega r_u, x_u += res, r_u -= res, push (1-alpha) res / d_u
 * (Katz: alpha res) as in ppr_sor (ppr_solver.py:331-461) / katz_sor
 * (katz_solver.py:251-337), in a Gauss-Seidel order the GPU can run in
 * parallel: sweeps over the colours of a greedy proper colouring (internal
 * degree-descending order), all pending nodes of one colour relaxing together.
 * A node is pending when an addition or its own update leaves |r_v| >=
 * eps_vec[v]; local = 1 stops after a sweep that leaves nothing pending,
 * local = 0 relaxes every node each sweep and stops when no node is at or
 * above threshold (oper += n + m per sweep).  The order differs from the
 * reference's FIFO queue, so operation counts differ from its (both meet the
 * same stopping rule).  p->kind GDE_PPR / GDE_KATZ, p->omega in (0, 2),
 * p->max_rounds caps the sweeps.  Outputs dense [nq][n] (ld_out = n). */
int gde_sor(gde_ctx *ctx, gde_graph *g, const gde_params *p, int64_t nq, const int32_t *seeds, const double *eps,
            int local, void *x_out, void *r_out, int out64, int out_mem, int64_t ld_out, double *oper_out,
            int32_t *sweeps_out, gde_stats *stats);
/* The colouring gde_sor uses, per caller node id (host colors_out[n], may be
 * NULL), and the number of colours. */
int gde_graph_colors(gde_graph *g, int32_t *colors_out, int32_t *ncolors);

/* ---- Katz Chebyshev spectral bounds ----
 * lambda_max(A) and lambda_min(A) of the graph's adjacency by a Lanczos
 * iteration on the GPU (FP64), the quantities katz_exp_dmax.py:20 and
 * katz_exp_dmin.py:20 obtain with scipy.sparse.linalg.eigsh; l_max =
 * 1 - alpha lambda_min and mu_min = 1 - alpha lambda_max bound the spectrum
 * of Q = I - alpha A for katz_cheby (katz_solver.py:340-368).  Stops when
 * both extreme Ritz values change by less than tol (relative) over 5 steps;
 * GDE_EITERCAP (with the last estimates written) after max_iter steps.
 * Outputs are host pointers (may be NULL). */
int gde_katz_spectral_bounds(gde_ctx *ctx, gde_graph *g, double alpha, int max_iter, double tol, double *lam_max,
                             double *lam_min, double *l_max, double *mu_min);

/* heat-kernel Taylor length, hk_solver.py:28-48 (estimate_n) */
int64_t gde_hk_estimate_n(double tau, double eps);

/* ---- multi-column feature push (InstantGNN) ----
 * P, R: device n x F matrices (row stride ld, FP64 if prec == GDE_FP64 else
 * FP32), updated in place.  Columns start with candidates = every node
 * (instantGNNParallel's initial scan, InstantGNN.py:59-63) when cand == NULL,
 * else the host list cand[0..ncand).  kind GDE_IGN: p += alpha r,
 * r_v += (1-alpha) r_u / d_u^(1-beta) / d_v^beta, threshold d^(1-beta) eps;
 * kind GDE_UPPR (beta = 0): p += r, threshold alpha eps d.  p->omega 0 or 1:
 * synchronous frontier push; otherwise res = omega r_u relaxes in
 * multicolour SOR order (as gde_sor; instantGNNSorPush, InstantGNN.py:74-105,
 * and update_ppr's push, ppr_solver.py:798-819), on padded graphs only.
 * Replaces instantGNNParallel / instantGNNSorParallel (InstantGNN.py:46-134);
 * oper_out (host, may be NULL) receives per-column operation counts. */
int gde_feature_push(gde_ctx *ctx, gde_graph *g, const gde_params *p, int64_t F, void *P, void *R, int64_t ld,
                     double eps, const int32_t *cand, int64_t ncand, double *oper_out, gde_stats *stats);

/* ---- dynamic graph update + incremental feature push ----
 * Applies the edge batch (us[i], vs[i]) to the padded CSR exactly as
 * updetaGraph does (InstantGNN.py:137-180; insertion only when only_insert,
 * else existing edges are deleted), mutating the caller's host arrays
 * h_indices / h_degree in place and the device copy of the graph; repairs
 * P, R at the touched nodes from X (InstantGNN.py:303-318, kind GDE_IGN) or
 * with the beta = 0 rule (ppr_solver.py:776-792, kind GDE_UPPR); then
 * pushes from the repaired nodes (with p->omega as gde_feature_push; the
 * colouring is rebuilt for the edited graph).  Replaces instantGNNUpdateBatchParallel
 * (InstantGNN.py:332-359) and update_ppr_parallel (ppr_solver.py:824-849).
 * X may be NULL for GDE_UPPR.  The whole edit runs on the device.  Before
 * anything is edited, an endpoint outside [0, n) or a graph uploaded with a
 * degree array that is not its row length gives GDE_EINVAL.  An edge that
 * fails stops the batch after the edges before it, which stay applied (in
 * the caller's arrays and on the device), and nothing is repaired or pushed:
 * an insertion into a row without slack gives GDE_ECAPACITY; a self-loop
 * insertion, which the reference writes into one slot while counting two
 * degrees, gives GDE_EINVAL when the second slot holds the padding sentinel
 * n (the next push would read it as a node id). */
int gde_feature_update(gde_ctx *ctx, gde_graph *g, int32_t *h_indices, int64_t *h_degree, const int32_t *us,
                       const int32_t *vs, int64_t k, int only_insert, const gde_params *p, int64_t F, void *P,
                       void *R, const void *X, int64_t ld, double eps, double *oper_out, gde_stats *stats);

/* ---- padded-CSR edge batch alone (updetaGraph / updeta_graph) ----
 * Applies the batch (us[i], vs[i]) exactly as updetaGraph (InstantGNN.py:137-180)
 * and updeta_graph (ppr_solver.py:723-766) do -- the edit gde_feature_update
 * starts with, on the device, without a repair or push -- mutating the
 * caller's host arrays h_indices / h_degree and the resident graph.
 * outcome (host, may be NULL): k bytes, per edge 0 = no change, 1 = inserted,
 * 2 = deleted, from which the caller rebuilds the reference's
 * insert_neighbor / delete_neighbor maps in batch order.  Errors as for
 * gde_feature_update: a row without slack stops the batch (GDE_ECAPACITY)
 * after the edges before it, as the sequential pass would.  stats (may be
 * NULL) gets edit_path and edit_ms. */
int gde_graph_update(gde_ctx *ctx, gde_graph *g, int32_t *h_indices, int64_t *h_degree, const int32_t *us,
                     const int32_t *vs, int64_t k, int only_insert, uint8_t *outcome, gde_stats *stats);

/* ---- repair of P, R after an edge batch (the first half of instantGNNUpdateBatch / update_ppr) ----
 * For each key u = keys[i] (a node with insertions), with its degree
 * old_degree[i] before the batch and its degree now from the resident
 * (edited) graph: rescales P[u], R[u] and adds the neighbour terms of its
 * inserted neighbours nbr[nbr_off[2i] .. nbr_off[2i+1]) minus those of its
 * deleted neighbours nbr[nbr_off[2i+1] .. nbr_off[2i+2]), for every column,
 * in the reference's arithmetic: kind GDE_IGN (InstantGNN.py:303-314, needs
 * X; pass no deleted neighbours when the reference's algo contains
 * 'insert') or GDE_UPPR (ppr_solver.py:776-792).  P, R, X: device n x F
 * matrices with row stride ld (FP64 if p->prec == GDE_FP64, else FP32).
 * keys, old_degree, nbr_off (2 nkeys + 1 entries), nbr: host arrays.  The push
 * from the repaired nodes is gde_feature_push with cand = keys. */
int gde_feature_repair(gde_ctx *ctx, gde_graph *g, const gde_params *p, int64_t F, void *P, void *R, const void *X,
                       int64_t ld, int64_t nkeys, const int32_t *keys, const int64_t *old_degree,
                       const int64_t *nbr_off, const int32_t *nbr);

/* Slack management for padded graphs (no counterpart in the reference, whose
 * padded layout is fixed when data_process_GNN.py:93-171 builds it).  Re-lays
 * the graph so every row has at least min_slack free slots after its live
 * entries; rows that already have that much keep their capacity.  Two calls:
 * with indices_out NULL it only writes the new capacity to *cap_out; then,
 * with indptr_out[n + 1] and indices_out[*cap_out], it moves the rows on the
 * device and writes the new host arrays (live entries first, slack filled
 * with the sentinel n).  Degrees, tables and the node ids are unchanged; the
 * caller's degree array stays valid.  A row without slack makes
 * gde_feature_update return GDE_ECAPACITY; this is the way to grow it. */
int gde_graph_repad(gde_ctx *ctx, gde_graph *g, int64_t min_slack, int64_t *indptr_out, int32_t *indices_out,
                    int64_t *cap_out);

/* ---- plain single-query baseline ----
 * The structure of ppr_gd_local_gpu (ppr_solver.py:82-146) on this GPU:
 * thread-per-row atomic kernel, O(n) passes and a host sync every round.
 * x_out / r_out: device FP32 [n] (may be NULL).  Benchmark denominator. */
int gde_plain_ppr_local(gde_ctx *ctx, gde_graph *g, int32_t seed, double alpha, double eps, float *x_out,
                        float *r_out, double *oper_out, int32_t *rounds_out);

/* ---- random-access ceiling (measurement) ----
 * No counterpart in the reference: the rate of uniformly random FP32
 * atomic adds (with_return != 0: with their return value, as the push's
 * crossing test uses them) over an array of n_floats entries, in G atomics/s
 * (best of three launches of 8 blocks x 256 threads per SM, 64 atomics per
 * thread).  The push kernel's residual scatter is bounded by this rate at its
 * slabs' size, not by streaming HBM bandwidth. */
int gde_probe_random_atomics(gde_ctx *ctx, int64_t n_floats, int with_return, double *gops_out);

/* ---- single-query solve that allocates no device memory ----
 * No counterpart in the reference: an addition of this library for callers
 * that must not allocate device memory while serving a request (a host that
 * owns all GPU memory through its own pool, a latency-bound loop where
 * cudaMalloc/cudaFree would synchronise the device, a process close to its
 * memory limit).  One PPR or Katz query (p->kind GDE_PPR / GDE_KATZ, p->method
 * GDE_LOCAL_GD / GDE_GLOBAL_GD, p->prec FP32 / FP64; same results as gde_solve
 * for that query) whose workspace is a fixed 64 MiB device array inside the
 * library: about 44 bytes per node in FP32 (52 in FP64) plus cap / 8 bytes;
 * larger graphs are rejected with GDE_EINVAL.  Calls no cudaMalloc, cudaFree
 * or other allocating routine.  Every call on a device shares the array, so
 * calls whose GPU work overlaps race: serialise them.  The first call on a
 * device looks the array up (cudaGetSymbolAddress); make it before any stream
 * capture.  x_out / r_out: device [n] in caller node order (FP64 if out64,
 * else FP32; may be NULL); oper_out / rounds_out: host (may be NULL). */
int gde_solve_noalloc(gde_ctx *ctx, gde_graph *g, const gde_params *p, int32_t seed, double eps, void *x_out,
                      void *r_out, int out64, double *oper_out, int32_t *rounds_out);

#ifdef __cplusplus
}
#endif

#endif /* GDE_H_ */
