/*
 * gde_oracle.c -- CPU restatement of the reference's local push solvers.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU library is
 * checked against and the timed CPU baseline of the benchmark; no product
 * code path links, loads or calls it.
 *
 * Every function restates one reference function (file:line given beside it)
 * in FP64 with the same order of floating-point operations, so that on the
 * same inputs it reproduces the reference's output bit for bit (pinned by the
 * golden fixtures generated from the reference itself).  Build with
 * -ffp-contract=off: a fused multiply-add would change the rounding.
 *
 * Besides the reference's own (sequential) semantics, the "sync" variants
 * restate the synchronous frontier rule the GPU kernels implement for
 * Chebyshev and InstantGNN pushes: the frontier of the next round is every
 * node whose residual passes its threshold after the round.  For local GD,
 * Katz GD and the heat-kernel level push (omega = 1) the reference's own rule
 * already is that set, so those need no separate variant.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t i64;
typedef int32_t i32;

/* ------------------------------------------------------------------------ */
/* PPR: ppr_gd (ppr_solver.py:208-328)                                        */
/* ------------------------------------------------------------------------ */
i64 orc_ppr_gd(i64 n, const i64 *indptr, const i32 *indices, const double *degree, i64 s, double alpha,
               double eps, int local, double *xt, double *rt) {
    double *tmp_rt = (double *)calloc((size_t)n, sizeof(double));
    double *eps_vec = (double *)malloc((size_t)n * sizeof(double));
    double m = 0.0;
    i64 oper = 0;
    memset(xt, 0, (size_t)n * sizeof(double));
    memset(rt, 0, (size_t)n * sizeof(double));
    rt[s] = alpha;
    for (i64 i = 0; i < n; i++) eps_vec[i] = eps * alpha * degree[i];
    for (i64 i = 0; i < n; i++) m += degree[i];
    if (local) {
        i64 *queue = (i64 *)calloc((size_t)n, sizeof(i64));
        i64 *st = (i64 *)calloc((size_t)n, sizeof(i64));
        unsigned char *q_mark = (unsigned char *)calloc((size_t)n, 1);
        queue[0] = s;
        q_mark[s] = 1;
        i64 rear = 1;
        for (;;) {
            for (i64 i = 0; i < rear; i++) oper += (i64)degree[queue[i]];
            if (rear == 0) break;
            if ((double)rear < (double)n / 4.0) {
                memcpy(st, queue, (size_t)rear * sizeof(i64));
            } else { /* np.nonzero(q_mark): ascending node order (:271-272) */
                i64 k = 0;
                for (i64 i = 0; i < n; i++)
                    if (q_mark[i]) st[k++] = i;
            }
            for (i64 i = 0; i < rear; i++) tmp_rt[i] = rt[st[i]];
            for (i64 i = 0; i < rear; i++) q_mark[st[i]] = 0;
            for (i64 i = 0; i < rear; i++) xt[st[i]] += tmp_rt[i];
            for (i64 i = 0; i < rear; i++) rt[st[i]] -= tmp_rt[i];
            i64 tmp_rear = rear;
            rear = 0;
            for (i64 ind = 0; ind < tmp_rear; ind++) {
                i64 u = st[ind];
                double val = (1. - alpha) * tmp_rt[ind] / degree[u];
                for (i64 j = indptr[u]; j < indptr[u + 1]; j++) {
                    i64 v = indices[j];
                    rt[v] += val;
                    if (!q_mark[v] && eps_vec[v] <= fabs(rt[v])) {
                        queue[rear++] = v;
                        q_mark[v] = 1;
                    }
                }
            }
        }
        free(queue);
        free(st);
        free(q_mark);
    } else {
        for (;;) {
            i64 cnt = 0;
            for (i64 i = 0; i < n; i++) cnt += (eps_vec[i] <= fabs(rt[i]));
            if (cnt <= 0) break;
            for (i64 i = 0; i < n; i++) xt[i] += rt[i];
            memset(tmp_rt, 0, (size_t)n * sizeof(double));
            for (i64 u = 0; u < n; u++) {
                double val = (1. - alpha) * rt[u] / degree[u];
                for (i64 j = indptr[u]; j < indptr[u + 1]; j++) tmp_rt[indices[j]] += val;
            }
            memcpy(rt, tmp_rt, (size_t)n * sizeof(double));
            oper += n + (i64)m;
        }
    }
    free(tmp_rt);
    free(eps_vec);
    return oper;
}

/* ------------------------------------------------------------------------ */
/* PPR / Katz Chebyshev: ppr_cheby (ppr_solver.py:582-661),                  */
/* katz_cheby (katz_solver.py:340-431).  katz=0: PPR, katz=1: Katz.         */
/* sync=1 replaces the in-sweep enqueue with the synchronous frontier rule.  */
/* ------------------------------------------------------------------------ */
i64 orc_cheby(i64 n, const i64 *indptr, const i32 *indices, const double *degree, i64 s, double alpha,
              double eps, int local, int katz, double l_max, double mu_min, int sync, double *xt, double *rt) {
    double *dx = (double *)calloc((size_t)n, sizeof(double));
    double *tmp_vec = (double *)calloc((size_t)n, sizeof(double));
    double *eps_vec = (double *)malloc((size_t)n * sizeof(double));
    double m = 0.0, delta_t, beta = 0, beta1 = 0, beta2 = 0;
    i64 oper = 0;
    for (i64 i = 0; i < n; i++) m += degree[i];
    memset(xt, 0, (size_t)n * sizeof(double));
    memset(rt, 0, (size_t)n * sizeof(double));
    if (!katz) {
        rt[s] = alpha;
        for (i64 i = 0; i < n; i++) xt[i] = rt[i];
        for (i64 i = 0; i < n; i++) dx[i] = xt[i];
        for (i64 i = 0; i < n; i++) eps_vec[i] = eps * alpha * degree[i];
        delta_t = (1. - alpha);
        double val = (1. - alpha) * rt[s] / degree[s];
        for (i64 j = indptr[s]; j < indptr[s + 1]; j++) tmp_vec[indices[j]] += val;
        memcpy(rt, tmp_vec, (size_t)n * sizeof(double));
    } else {
        xt[s] = 2. / (l_max + mu_min);
        for (i64 i = 0; i < n; i++) dx[i] = xt[i];
        rt[s] = 1. - 2. / (l_max + mu_min);
        double val = 2. * alpha / (l_max + mu_min);
        for (i64 j = indptr[s]; j < indptr[s + 1]; j++) rt[indices[j]] += val;
        for (i64 i = 0; i < n; i++) eps_vec[i] = eps * degree[i];
        delta_t = (l_max - mu_min) / (l_max + mu_min);
    }
    if (!local) {
        for (;;) {
            i64 cnt = 0;
            for (i64 i = 0; i < n; i++) cnt += (eps_vec[i] <= fabs(rt[i]));
            if (cnt <= 0) break;
            oper += n + (i64)m;
            if (!katz) {
                delta_t = 1. / (2. / (1. - alpha) - delta_t);
                beta = 2. * delta_t / (1. - alpha);
                for (i64 i = 0; i < n; i++) tmp_vec[i] = beta * rt[i] + (beta - 1.) * dx[i];
            } else {
                delta_t = 1. / (2. * ((l_max + mu_min) / (l_max - mu_min)) - delta_t);
                beta1 = 4. * delta_t / (l_max - mu_min);
                beta2 = (1. - 2. * delta_t * (l_max + mu_min) / (l_max - mu_min));
                for (i64 i = 0; i < n; i++) tmp_vec[i] = beta1 * rt[i] - beta2 * dx[i];
            }
            for (i64 i = 0; i < n; i++) xt[i] += tmp_vec[i];
            memcpy(dx, tmp_vec, (size_t)n * sizeof(double));
            memset(tmp_vec, 0, (size_t)n * sizeof(double));
            for (i64 u = 0; u < n; u++) {
                double val = katz ? alpha * dx[u] : (1. - alpha) * dx[u] / degree[u];
                for (i64 j = indptr[u]; j < indptr[u + 1]; j++) tmp_vec[indices[j]] += val;
            }
            if (!katz)
                for (i64 i = 0; i < n; i++) rt[i] += tmp_vec[i] - dx[i];
            else
                for (i64 i = 0; i < n; i++) rt[i] = rt[i] + tmp_vec[i] - dx[i];
        }
    } else {
        i64 *queue = (i64 *)calloc((size_t)n, sizeof(i64));
        i64 *queue_pre = (i64 *)calloc((size_t)n, sizeof(i64));
        unsigned char *q_mark = (unsigned char *)calloc((size_t)n, 1);
        i64 rear = 0;
        if (sync && eps_vec[s] <= fabs(rt[s])) { /* the sync rule also tests the seed itself */
            queue[rear++] = s;
            q_mark[s] = 1;
        }
        for (i64 j = indptr[s]; j < indptr[s + 1]; j++) {
            i64 v = indices[j];
            if (!q_mark[v] && eps_vec[v] <= fabs(rt[v])) {
                queue[rear++] = v;
                q_mark[v] = 1;
            }
        }
        for (;;) {
            if (sync && rear > 0) {
                /* the sync rule marks without filling queue[]: rebuild it first */
                i64 k = 0;
                for (i64 i = 0; i < n; i++)
                    if (q_mark[i]) queue[k++] = i;
            }
            if (katz)
                for (i64 i = 0; i < rear; i++) oper += (i64)degree[queue[i]];
            if (rear == 0) break;
            if (!katz)
                for (i64 i = 0; i < rear; i++) oper += (i64)degree[queue[i]];
            if (!katz) {
                delta_t = 1. / (2. / (1. - alpha) - delta_t);
                beta = 2. * delta_t / (1. - alpha);
            } else {
                delta_t = 1. / (2. * ((l_max + mu_min) / (l_max - mu_min)) - delta_t);
                beta1 = 4. * delta_t / (l_max - mu_min);
                beta2 = (1. - 2. * delta_t * (l_max + mu_min) / (l_max - mu_min));
            }
            if (sync || (double)rear > (double)n / 4.0) {
                /* ascending node order (:639-640); the sync rule always uses it */
                i64 k = 0;
                for (i64 i = 0; i < n; i++)
                    if (q_mark[i]) queue[k++] = i;
            }
            for (i64 ind = 0; ind < rear; ind++) {
                i64 u = queue[ind];
                double tmp = katz ? beta1 * rt[u] - beta2 * dx[u] : beta * rt[u] + (beta - 1.) * dx[u];
                xt[u] += tmp;
                dx[u] = tmp;
                q_mark[u] = 0;
                queue_pre[ind] = u;
            }
            i64 rear_pre = rear;
            rear = 0;
            for (i64 ind = 0; ind < rear_pre; ind++) {
                i64 u = queue_pre[ind];
                double val = katz ? alpha * dx[u] : (1. - alpha) * dx[u] / degree[u];
                for (i64 j = indptr[u]; j < indptr[u + 1]; j++) {
                    i64 v = indices[j];
                    rt[v] += val;
                    if (!sync && !q_mark[v] && eps_vec[v] <= fabs(rt[v])) {
                        queue[rear++] = v;
                        q_mark[v] = 1;
                    }
                }
                rt[u] += -dx[u];
            }
            if (sync) {
                /* next frontier: every node touched this round whose residual passes */
                for (i64 ind = 0; ind < rear_pre; ind++) {
                    i64 u = queue_pre[ind];
                    if (!q_mark[u] && eps_vec[u] <= fabs(rt[u])) { q_mark[u] = 1; rear++; }
                    for (i64 j = indptr[u]; j < indptr[u + 1]; j++) {
                        i64 v = indices[j];
                        if (!q_mark[v] && eps_vec[v] <= fabs(rt[v])) { q_mark[v] = 1; rear++; }
                    }
                }
            }
        }
        free(queue);
        free(queue_pre);
        free(q_mark);
    }
    free(dx);
    free(tmp_vec);
    free(eps_vec);
    return oper;
}

/* ------------------------------------------------------------------------ */
/* Katz GD: katz_gd (katz_solver.py:167-248)                                 */
/* ------------------------------------------------------------------------ */
i64 orc_katz_gd(i64 n, const i64 *indptr, const i32 *indices, const double *degree, i64 s, double alpha,
                double eps, int local, double *xt, double *rt) {
    double *tmp_rt = (double *)calloc((size_t)n, sizeof(double));
    double *eps_vec = (double *)malloc((size_t)n * sizeof(double));
    double m = 0.0;
    i64 oper = 0;
    memset(xt, 0, (size_t)n * sizeof(double));
    memset(rt, 0, (size_t)n * sizeof(double));
    rt[s] = 1.;
    for (i64 i = 0; i < n; i++) eps_vec[i] = eps * degree[i];
    for (i64 i = 0; i < n; i++) m += degree[i];
    if (local) {
        i64 *queue = (i64 *)calloc((size_t)n, sizeof(i64));
        i64 *st = (i64 *)calloc((size_t)n, sizeof(i64));
        unsigned char *q_mark = (unsigned char *)calloc((size_t)n, 1);
        queue[0] = s;
        q_mark[s] = 1;
        i64 rear = 1;
        for (;;) {
            for (i64 i = 0; i < rear; i++) oper += (i64)degree[queue[i]];
            if (rear == 0) break;
            if ((double)rear < (double)n / 4.0) {
                memcpy(st, queue, (size_t)rear * sizeof(i64));
            } else {
                i64 k = 0;
                for (i64 i = 0; i < n; i++)
                    if (q_mark[i]) st[k++] = i;
            }
            for (i64 i = 0; i < rear; i++) tmp_rt[i] = rt[st[i]];
            for (i64 i = 0; i < rear; i++) q_mark[st[i]] = 0;
            for (i64 i = 0; i < rear; i++) xt[st[i]] += tmp_rt[i];
            for (i64 i = 0; i < rear; i++) rt[st[i]] -= tmp_rt[i];
            i64 tmp_rear = rear;
            rear = 0;
            for (i64 ind = 0; ind < tmp_rear; ind++) {
                i64 u = st[ind];
                double val = alpha * tmp_rt[ind];
                for (i64 j = indptr[u]; j < indptr[u + 1]; j++) {
                    i64 v = indices[j];
                    rt[v] += val;
                    if (!q_mark[v] && eps_vec[v] <= fabs(rt[v])) {
                        queue[rear++] = v;
                        q_mark[v] = 1;
                    }
                }
            }
        }
        free(queue);
        free(st);
        free(q_mark);
    } else {
        for (;;) {
            i64 cnt = 0;
            for (i64 i = 0; i < n; i++) cnt += (eps_vec[i] <= fabs(rt[i]));
            if (cnt <= 0) break;
            for (i64 i = 0; i < n; i++) xt[i] += rt[i];
            memset(tmp_rt, 0, (size_t)n * sizeof(double));
            for (i64 u = 0; u < n; u++) {
                double val = alpha * rt[u];
                for (i64 j = indptr[u]; j < indptr[u + 1]; j++) tmp_rt[indices[j]] += val;
            }
            memcpy(rt, tmp_rt, (size_t)n * sizeof(double));
            oper += n + (i64)m;
        }
    }
    xt[s] -= 1.;
    free(tmp_rt);
    free(eps_vec);
    return oper;
}

/* ------------------------------------------------------------------------ */
/* SOR / APPR: ppr_sor (ppr_solver.py:331-461), katz_sor (katz_solver.py:251- */
/* 337).  Neighbour slice is indices[indptr[u] : indptr[u]+degree[u]].       */
/* ------------------------------------------------------------------------ */
double orc_sor(i64 n, const i64 *indptr, const i32 *indices, const double *degree, i64 s, double alpha,
               double eps, double omega, int local, int katz, double *xt, double *rt) {
    double *eps_vec = (double *)malloc((size_t)n * sizeof(double));
    double m = 0.0, oper = 0.;
    for (i64 i = 0; i < n; i++) m += degree[i];
    memset(xt, 0, (size_t)n * sizeof(double));
    memset(rt, 0, (size_t)n * sizeof(double));
    rt[s] = katz ? 1.0 : alpha;
    for (i64 i = 0; i < n; i++) eps_vec[i] = katz ? eps * degree[i] : eps * alpha * degree[i];
    if (local) {
        i64 q_max = n + 2, front = 0, rear = 0;
        i64 *queue = (i64 *)calloc((size_t)q_max, sizeof(i64));
        unsigned char *q_mark = (unsigned char *)calloc((size_t)q_max, 1);
        queue[rear] = n;
        rear = (rear + 1) % q_max;
        q_mark[n] = 1;
        queue[rear] = s;
        rear = (rear + 1) % q_max;
        q_mark[s] = 1;
        for (;;) {
            i64 u = queue[front];
            front = (front + 1) % q_max;
            q_mark[u] = 0;
            if (u == n) {
                if ((rear - front) == 0) break;
                queue[rear] = n;
                rear = (rear + 1) % q_max;
                q_mark[u] = 1;
                continue;
            }
            if (eps_vec[u] > fabs(rt[u])) continue;
            oper += degree[u];
            double res = omega * rt[u];
            xt[u] += res;
            rt[u] -= res;
            double push_res = katz ? alpha * res : (1. - alpha) * res / degree[u];
            i64 end = katz ? indptr[u + 1] : indptr[u] + (i64)degree[u];
            for (i64 j = indptr[u]; j < end; j++) {
                i64 v = indices[j];
                rt[v] += push_res;
                if (!q_mark[v] && eps_vec[v] <= fabs(rt[v])) {
                    queue[rear] = v;
                    rear = (rear + 1) % q_max;
                    q_mark[v] = 1;
                }
            }
            if (!q_mark[u] && eps_vec[u] <= fabs(rt[u])) {
                queue[rear] = u;
                rear = (rear + 1) % q_max;
                q_mark[u] = 1;
            }
        }
        free(queue);
        free(q_mark);
    } else {
        for (;;) {
            for (i64 u = 0; u < n; u++) {
                double res = omega * rt[u];
                xt[u] += res;
                rt[u] -= res;
                double push_res = katz ? alpha * res : (1. - alpha) * res / degree[u];
                i64 end = katz ? indptr[u + 1] : indptr[u] + (i64)degree[u];
                for (i64 j = indptr[u]; j < end; j++) rt[indices[j]] += push_res;
            }
            oper += (double)n + m;
            i64 cnt = 0;
            for (i64 i = 0; i < n; i++) cnt += (eps_vec[i] <= fabs(rt[i]));
            if (cnt <= 0) break;
        }
    }
    if (katz) xt[s] -= 1.;
    free(eps_vec);
    return oper;
}

/* ------------------------------------------------------------------------ */
/* Multicolour local / global SOR: the parallel order of the GPU LocalSOR.   */
/* The update of a node is ppr_sor's (ppr_solver.py:390-402; katz_sor,       */
/* katz_solver.py:296-310): res = omega r_u, x_u += res, r_u -= res, push    */
/* (1-alpha) res / d_u (Katz: alpha res) to every neighbour.  The order is   */
/* a sweep over colours c = 0..C-1 of a proper colouring; in colour c's      */
/* phase every pending node of colour c with |r_u| >= eps_vec[u] relaxes.   */
/* Same-coloured nodes are not adjacent, so a phase equals a sequential     */
/* Gauss-Seidel pass over them in any order.  A node becomes pending when   */
/* an addition leaves |r_v| >= eps_vec[v] (the reference's enqueue test,    */
/* :398-401), or when its own update leaves it there (:402-405); it is      */
/* processed at the next phase of its colour.  Local stops after a sweep    */
/* that leaves nothing pending; global relaxes every node of each colour    */
/* and stops after a sweep with no node at or above threshold (:452-457).   */
/* ------------------------------------------------------------------------ */
double orc_sor_color(i64 n, const i64 *indptr, const i32 *indices, const double *degree, i64 s, double alpha,
                     double eps, double omega, int local, int katz, const i32 *color, i64 ncolors, double *xt,
                     double *rt, i64 *sweeps_out) {
    double *eps_vec = (double *)malloc((size_t)n * sizeof(double));
    double m = 0.0, oper = 0.;
    for (i64 i = 0; i < n; i++) m += degree[i];
    memset(xt, 0, (size_t)n * sizeof(double));
    memset(rt, 0, (size_t)n * sizeof(double));
    rt[s] = katz ? 1.0 : alpha;
    for (i64 i = 0; i < n; i++) eps_vec[i] = katz ? eps * degree[i] : eps * alpha * degree[i];
    /* nodes of each colour, in node order */
    i64 *cstart = (i64 *)calloc((size_t)ncolors + 1, sizeof(i64));
    i64 *corder = (i64 *)malloc((size_t)(n > 0 ? n : 1) * sizeof(i64));
    for (i64 i = 0; i < n; i++) cstart[color[i] + 1]++;
    for (i64 c = 0; c < ncolors; c++) cstart[c + 1] += cstart[c];
    {
        i64 *fill = (i64 *)calloc((size_t)ncolors, sizeof(i64));
        for (i64 i = 0; i < n; i++) corder[cstart[color[i]] + fill[color[i]]++] = i;
        free(fill);
    }
    i64 sweeps = 0;
    if (local) {
        /* pending lists per colour (capacity: the colour's node count) */
        i64 *plist = (i64 *)malloc((size_t)(n > 0 ? n : 1) * sizeof(i64));
        i64 *pcnt = (i64 *)calloc((size_t)ncolors, sizeof(i64));
        i64 *cur = (i64 *)malloc((size_t)(n > 0 ? n : 1) * sizeof(i64));
        unsigned char *mark = (unsigned char *)calloc((size_t)(n > 0 ? n : 1), 1);
        plist[cstart[color[s]]] = s;
        pcnt[color[s]] = 1;
        mark[s] = 1;
        for (;;) {
            i64 pend = 0;
            for (i64 c = 0; c < ncolors; c++) pend += pcnt[c];
            if (pend == 0) break;
            sweeps++;
            for (i64 c = 0; c < ncolors; c++) {
                i64 k = pcnt[c];
                if (k == 0) continue;
                memcpy(cur, plist + cstart[c], (size_t)k * sizeof(i64));
                pcnt[c] = 0;
                for (i64 i = 0; i < k; i++) mark[cur[i]] = 0;
                for (i64 i = 0; i < k; i++) {
                    i64 u = cur[i];
                    if (eps_vec[u] > fabs(rt[u])) continue;
                    oper += degree[u];
                    double res = omega * rt[u];
                    xt[u] += res;
                    rt[u] -= res;
                    double push_res = katz ? alpha * res : (1. - alpha) * res / degree[u];
                    i64 end = katz ? indptr[u + 1] : indptr[u] + (i64)degree[u];
                    for (i64 j = indptr[u]; j < end; j++) {
                        i64 v = indices[j];
                        rt[v] += push_res;
                        if (!mark[v] && eps_vec[v] <= fabs(rt[v])) {
                            mark[v] = 1;
                            plist[cstart[color[v]] + pcnt[color[v]]++] = v;
                        }
                    }
                    if (!mark[u] && eps_vec[u] <= fabs(rt[u])) {
                        mark[u] = 1;
                        plist[cstart[c] + pcnt[c]++] = u;
                    }
                }
            }
        }
        free(plist);
        free(pcnt);
        free(cur);
        free(mark);
    } else {
        for (;;) {
            sweeps++;
            for (i64 c = 0; c < ncolors; c++) {
                for (i64 i = cstart[c]; i < cstart[c + 1]; i++) {
                    i64 u = corder[i];
                    double res = omega * rt[u];
                    if (res == 0.0) continue;
                    xt[u] += res;
                    rt[u] -= res;
                    double push_res = katz ? alpha * res : (1. - alpha) * res / degree[u];
                    i64 end = katz ? indptr[u + 1] : indptr[u] + (i64)degree[u];
                    for (i64 j = indptr[u]; j < end; j++) rt[indices[j]] += push_res;
                }
            }
            oper += (double)n + m;
            i64 cnt = 0;
            for (i64 i = 0; i < n; i++) cnt += (eps_vec[i] <= fabs(rt[i]));
            if (cnt <= 0) break;
        }
    }
    if (katz) xt[s] -= 1.;
    if (sweeps_out) *sweeps_out = sweeps;
    free(eps_vec);
    free(cstart);
    free(corder);
    return oper;
}

/* Multicolour SOR push of one InstantGNN column (the GPU order for          */
/* instantGNNSorPush, InstantGNN.py:74-105): sweeps over colours; in colour  */
/* c's phase every pending node of colour c with |r_u| >= eps_vec[u]         */
/* relaxes -- absorbing nodes take p = r, r = 0; others res = omega r_u,     */
/* p += alpha res, r_u = (1-omega) r_u, r_v += (1-alpha) res / d_u^(1-beta)  */
/* / d_v^beta.  Pending: the candidates at or above threshold at the start, */
/* then every node an addition or its own update leaves there.  p, r have   */
/* stride cs.  Returns the sum of degrees of the relaxed non-absorbing      */
/* nodes.  uppr=1 gives update_ppr's push instead (ppr_solver.py:806-813):  */
/* p += res, r_u -= res, r_v += (1-alpha) res / d_u.                        */
i64 orc_ign_sor_color_column(i64 n, const i64 *indptr, const i32 *indices, const i64 *degree, double alpha,
                             const double *eps_vec, double beta, double omega, double *p, double *r, i64 cs,
                             const unsigned char *cand0, const i32 *color, i64 ncolors, int uppr) {
    i64 *cstart = (i64 *)calloc((size_t)ncolors + 1, sizeof(i64));
    for (i64 i = 0; i < n; i++) cstart[color[i] + 1]++;
    for (i64 c = 0; c < ncolors; c++) cstart[c + 1] += cstart[c];
    i64 *plist = (i64 *)malloc((size_t)(n > 0 ? n : 1) * sizeof(i64));
    i64 *pcnt = (i64 *)calloc((size_t)ncolors, sizeof(i64));
    i64 *cur = (i64 *)malloc((size_t)(n > 0 ? n : 1) * sizeof(i64));
    unsigned char *mark = (unsigned char *)calloc((size_t)(n > 0 ? n : 1), 1);
    i64 oper = 0;
    for (i64 u = 0; u < n; u++)
        if (cand0[u] && fabs(r[u * cs]) >= eps_vec[u]) {
            mark[u] = 1;
            plist[cstart[color[u]] + pcnt[color[u]]++] = u;
        }
    for (;;) {
        i64 pend = 0;
        for (i64 c = 0; c < ncolors; c++) pend += pcnt[c];
        if (pend == 0) break;
        for (i64 c = 0; c < ncolors; c++) {
            i64 k = pcnt[c];
            if (k == 0) continue;
            memcpy(cur, plist + cstart[c], (size_t)k * sizeof(i64));
            pcnt[c] = 0;
            for (i64 i = 0; i < k; i++) mark[cur[i]] = 0;
            for (i64 i = 0; i < k; i++) {
                i64 u = cur[i];
                double ru = r[u * cs];
                if (fabs(ru) < eps_vec[u]) continue;
                if ((degree[u] == 1 && indices[indptr[u]] == u) || degree[u] == 0) {
                    p[u * cs] = ru;
                    r[u * cs] = 0;
                    continue;
                }
                oper += degree[u];
                double res_u = omega * ru;
                double push_u;
                if (uppr) {  /* ppr_solver.py:806-809 */
                    p[u * cs] += res_u;
                    push_u = (1. - alpha) * res_u / (double)degree[u];
                    r[u * cs] -= res_u;
                } else {
                    p[u * cs] += alpha * res_u;
                    push_u = (1. - alpha) * res_u / pow((double)degree[u], 1 - beta);
                    r[u * cs] = (1 - omega) * ru;
                }
                for (i64 e = indptr[u]; e < indptr[u] + degree[u]; e++) {
                    i64 v = indices[e];
                    r[v * cs] += uppr ? push_u : push_u / pow((double)degree[v], beta);
                    if (!mark[v] && fabs(r[v * cs]) >= eps_vec[v]) {
                        mark[v] = 1;
                        plist[cstart[color[v]] + pcnt[color[v]]++] = v;
                    }
                }
                if (!mark[u] && fabs(r[u * cs]) >= eps_vec[u]) {
                    mark[u] = 1;
                    plist[cstart[c] + pcnt[c]++] = u;
                }
            }
        }
    }
    free(cstart);
    free(plist);
    free(pcnt);
    free(cur);
    free(mark);
    return oper;
}

/* ------------------------------------------------------------------------ */
/* Heat kernel (hk_solver.py:15-80, :206-295)                                */
/* ------------------------------------------------------------------------ */
static double est_coef(double t, i64 k) { /* estimate_coefficient, :15-25 */
    double t0 = t;
    if (k == 0) return t0;
    for (i64 i = 0; i < k; i++) t0 = t0 * (t / (double)(i + 2));
    return t0;
}

i64 orc_hk_estimate_n(double t, double eps) { /* estimate_n, :28-48 */
    double kf = ceil(t - 1);
    i64 k = (i64)kf;
    double cur_est = est_coef(t, k) * ((kf + 2.) / (kf + 2. - t));
    if (cur_est < eps * exp(t)) return k;
    i64 est_k = k;
    for (i64 i = k; i < 1000 * (k + 1); i++) {
        double tmp = ((kf + 2. - t) * t / pow(kf + 2., 2.)) * ((kf + 3.) / (kf + 3. - t));
        cur_est = cur_est * tmp;
        est_k += 1;
        if (cur_est < eps * exp(t)) return est_k;
    }
    return est_k;
}

/* hk_sor_queue, :206-295.  r2 receives the final [2, n] residual levels.    */
double orc_hk_sor_queue(i64 n, const i64 *indptr, const i32 *indices, const double *degree, i64 s, double tau,
                        double eps, double omega, int local, double *xt, double *r2, i64 *est_n_out) {
    double m = 0.0, oper = 0.;
    for (i64 i = 0; i < n; i++) m += degree[i];
    memset(xt, 0, (size_t)n * sizeof(double));
    memset(r2, 0, (size_t)(2 * n) * sizeof(double));
    double *rt[2] = {r2, r2 + n};
    i64 *queue[2];
    unsigned char *q_mark[2];
    for (int q = 0; q < 2; q++) {
        queue[q] = (i64 *)calloc((size_t)n, sizeof(i64));
        q_mark[q] = (unsigned char *)calloc((size_t)n, 1);
    }
    i64 rear[2] = {1, 0}, front[2] = {0, 0};
    queue[0][0] = s;
    q_mark[0][s] = 1;
    rt[0][s] = 1.;
    i64 est_n = orc_hk_estimate_n(tau, .5 * eps);
    double *psi = (double *)calloc((size_t)est_n + 1, sizeof(double));
    psi[est_n] = 1.;
    for (i64 i = est_n - 1; i >= 0; i--) psi[i] = psi[i + 1] * tau / ((double)i + 1.) + 1.;
    double *eps_vec = (double *)malloc((size_t)n * sizeof(double));
    for (i64 i = 0; i < n; i++) eps_vec[i] = exp(tau) * eps * degree[i] / (double)est_n;
    for (i64 j = 0; j < est_n; j++) {
        int qc = (int)(j % 2), qn = (int)((j + 1) % 2);
        if (local) {
            if (rear[qc] == front[qc]) break;
            while (front[qc] != rear[qc]) {
                i64 uu = queue[qc][front[qc] % n];
                front[qc] += 1;
                if (fabs(rt[qc][uu]) < eps_vec[uu] / psi[j]) continue;
                oper += degree[uu];
                double ru_j = omega * rt[qc][uu];
                xt[uu] += ru_j;
                rt[qc][uu] -= ru_j;
                double mass = (tau / ((double)j + 1.)) * ru_j / degree[uu];
                for (i64 e = indptr[uu]; e < indptr[uu + 1]; e++) {
                    i64 vv = indices[e];
                    if (j + 1 == est_n) {
                        xt[vv] += ru_j / degree[uu];
                        continue;
                    }
                    rt[qn][vv] = rt[qn][vv] + mass;
                    if (fabs(rt[qn][vv]) >= eps_vec[vv] / psi[j + 1] && !q_mark[qn][vv]) {
                        q_mark[qn][vv] = 1;
                        queue[qn][rear[qn]] = vv;
                        rear[qn] += 1;
                    }
                }
                if (fabs(rt[qc][uu]) >= eps_vec[uu] / psi[j] && !q_mark[qn][uu]) {
                    queue[qc][rear[qc] % n] = uu;
                    rear[qc] += 1;
                }
            }
        } else {
            for (;;) {
                for (i64 uu = 0; uu < n; uu++) {
                    double ru_j = omega * rt[qc][uu];
                    xt[uu] += ru_j;
                    rt[qc][uu] -= ru_j;
                    double mass = (tau / ((double)j + 1.)) * ru_j / degree[uu];
                    for (i64 e = indptr[uu]; e < indptr[uu + 1]; e++) {
                        i64 vv = indices[e];
                        if (j + 1 == est_n)
                            xt[vv] += ru_j / degree[uu];
                        else
                            rt[qn][vv] = rt[qn][vv] + mass;
                    }
                }
                oper += m + (double)n;
                i64 cnt = 0;
                for (i64 i = 0; i < n; i++) cnt += ((eps_vec[i] / psi[j]) <= fabs(rt[qc][i]));
                if (cnt <= 0) break;
            }
        }
        front[qc] = 0;
        rear[qc] = 0;
        memset(rt[qc], 0, (size_t)n * sizeof(double));
        memset(q_mark[qc], 0, (size_t)n);
    }
    double et = exp(tau);
    for (i64 i = 0; i < n; i++) xt[i] /= et;
    for (int q = 0; q < 2; q++) {
        free(queue[q]);
        free(q_mark[q]);
    }
    free(psi);
    free(eps_vec);
    *est_n_out = est_n;
    return oper;
}

/* Level-synchronous form of hk_sor_queue (the GPU's order).  Level j
 * pushes every node whose residual is at or above its threshold, each with
 * its relaxation sub-pushes back to back (omega r moved, r - omega r kept,
 * while the kept part stays at or above the threshold), in node order.
 * Without a queue there is no re-enqueue test on the next level's mark
 * (hk_solver.py:262), the only order-dependent step of the reference's local
 * form.  The global form is the reference's (:266-280): all nodes sweep
 * together until no residual is at or above threshold, so each node takes
 * the largest sub-push count any node needs. */
static double hk_relax_moved(double r, double omega, double thr, i64 fixed, i64 *subs, double *left) {
    double moved = 0.;
    i64 k = 0;
    do {
        double ru = omega * r;
        moved += ru;
        r -= ru;
        k++;
    } while (k < 65536 && (fixed > 0 ? k < fixed : fabs(r) >= thr));
    *subs = k;
    *left = r;
    return moved;
}

double orc_hk_sor_sync(i64 n, const i64 *indptr, const i32 *indices, const double *degree, i64 s, double tau,
                       double eps, double omega, int local, double *xt, double *r2, i64 *est_n_out) {
    double m = 0.0, oper = 0.;
    for (i64 i = 0; i < n; i++) m += degree[i];
    memset(xt, 0, (size_t)n * sizeof(double));
    memset(r2, 0, (size_t)(2 * n) * sizeof(double));
    double *rt[2] = {r2, r2 + n};
    rt[0][s] = 1.;
    i64 est_n = orc_hk_estimate_n(tau, .5 * eps);
    double *psi = (double *)calloc((size_t)est_n + 1, sizeof(double));
    psi[est_n] = 1.;
    for (i64 i = est_n - 1; i >= 0; i--) psi[i] = psi[i + 1] * tau / ((double)i + 1.) + 1.;
    double *eps_vec = (double *)malloc((size_t)n * sizeof(double));
    for (i64 i = 0; i < n; i++) eps_vec[i] = exp(tau) * eps * degree[i] / (double)est_n;
    for (i64 j = 0; j < est_n; j++) {
        double *rc = rt[j % 2], *rn = rt[(j + 1) % 2];
        i64 sweeps = 0, any = 0;
        for (i64 u = 0; u < n; u++) {
            double thr = eps_vec[u] / psi[j];
            if (fabs(rc[u]) >= thr) any = 1;
            if (!local) {
                i64 k;
                double left;
                hk_relax_moved(rc[u], omega, thr, 0, &k, &left);
                if (k > sweeps) sweeps = k;
            }
        }
        if (local && !any) break;
        for (i64 u = 0; u < n; u++) {
            double thr = eps_vec[u] / psi[j];
            if (local ? fabs(rc[u]) < thr : rc[u] == 0.) continue;
            i64 k;
            double left;
            double moved = hk_relax_moved(rc[u], omega, thr, local ? 0 : sweeps, &k, &left);
            if (local) oper += (double)k * degree[u];
            xt[u] += moved;
            rc[u] = left;
            for (i64 e = indptr[u]; e < indptr[u + 1]; e++) {
                i64 v = indices[e];
                if (j + 1 == est_n)
                    xt[v] += moved / degree[u];
                else
                    rn[v] += ((tau / ((double)j + 1.)) * moved) / degree[u];
            }
        }
        if (!local) oper += (double)sweeps * (m + (double)n);
        memset(rc, 0, (size_t)n * sizeof(double));
    }
    double et = exp(tau);
    for (i64 i = 0; i < n; i++) xt[i] /= et;
    free(psi);
    free(eps_vec);
    *est_n_out = est_n;
    return oper;
}

/* hk_taylor_approx, :51-80 */
i64 orc_hk_taylor(i64 n, const i64 *indptr, const i32 *indices, const double *degree, i64 s, double tau,
                  double eps, double *xt) {
    i64 est_n = orc_hk_estimate_n(tau, eps);
    double *cur = (double *)calloc((size_t)n, sizeof(double));
    double *tmp = (double *)calloc((size_t)n, sizeof(double));
    cur[s] = 1.;
    for (i64 i = 0; i < n; i++) xt[i] = 0.0 + cur[i];
    for (i64 k = 0; k < est_n; k++) {
        memset(tmp, 0, (size_t)n * sizeof(double));
        for (i64 u = 0; u < n; u++) {
            double val = cur[u] / degree[u];
            for (i64 e = indptr[u]; e < indptr[u + 1]; e++) tmp[indices[e]] += val;
        }
        double c = tau / ((double)k + 1.);
        for (i64 i = 0; i < n; i++) cur[i] = c * tmp[i];
        for (i64 i = 0; i < n; i++) xt[i] = xt[i] + cur[i];
    }
    double et = exp(tau);
    for (i64 i = 0; i < n; i++) xt[i] = xt[i] / et;
    free(cur);
    free(tmp);
    return est_n;
}

/* ------------------------------------------------------------------------ */
/* InstantGNN (InstantGNN.py:12-134).  Padded CSR: live neighbours of u are  */
/* indices[indptr[u] : indptr[u]+degree[u]].  p is float32 when p32 != NULL  */
/* (instantGNNParallel allocates p as float32, :55), else float64.          */
/* qn is the circular queue modulus (n+2 from the callers).                  */
/* ------------------------------------------------------------------------ */
static i64 ign_push(i64 qn, const i64 *indptr, const i32 *indices, const i64 *degree, double alpha,
                    const double *eps_vec, double omega, int sor, float *p32, double *p64, double *r,
                    i64 *queue, i64 front, i64 rear, unsigned char *q_mark, double beta) {
    /* returns the work done, sum of degree[u] over the pushes (the reference
     * does not count it; this is the count the synchronous form reports) */
    i64 oper = 0;
    while (rear != front) {
        front = (front + 1) % qn;
        i64 u = queue[front];
        q_mark[u] = 0;
        if (fabs(r[u]) < eps_vec[u]) continue;
        if ((degree[u] == 1 && indices[indptr[u]] == u) || degree[u] == 0) {
            if (p32) p32[u] = (float)r[u]; else p64[u] = r[u];
            r[u] = 0;
            continue;
        }
        double res_u = sor ? omega * r[u] : r[u];
        if (p32) p32[u] = (float)((double)p32[u] + alpha * res_u); else p64[u] += alpha * res_u;
        double push_u = (1. - alpha) * res_u / pow((double)degree[u], 1 - beta);
        oper += degree[u];
        r[u] = sor ? (1 - omega) * r[u] : 0;
        for (i64 e = indptr[u]; e < indptr[u] + degree[u]; e++) {
            i64 v = indices[e];
            r[v] += push_u / pow((double)degree[v], beta);
            if (!q_mark[v] && fabs(r[v]) >= eps_vec[v]) {
                rear = (rear + 1) % qn;
                queue[rear] = v;
                q_mark[v] = 1;
            }
        }
        if (!q_mark[u] && fabs(r[u]) >= eps_vec[u]) {
            rear = (rear + 1) % qn;
            queue[rear] = u;
            q_mark[u] = 1;
        }
    }
    return oper;
}

/* instantGNNParallel / instantGNNSorParallel for one column (:46-71, :108-134).
 * r (stride rs) is updated in place; p receives the propagated column.
 * Returns the push's work (sum of degree[u] over the pushes). */
i64 orc_ign_static_column(i64 n, const i64 *indptr, const i32 *indices, const i64 *degree, double alpha,
                           double eps, double omega, int sor, double beta, double *p_out, i64 ps, double *r,
                           i64 rs) {
    double *eps_vec = (double *)malloc((size_t)n * sizeof(double));
    double *rc = (double *)malloc((size_t)n * sizeof(double));
    i64 *queue = (i64 *)calloc((size_t)n + 2, sizeof(i64));
    unsigned char *q_mark = (unsigned char *)calloc((size_t)n, 1);
    for (i64 i = 0; i < n; i++) eps_vec[i] = pow((double)degree[i], 1 - beta) * eps;
    for (i64 i = 0; i < n; i++) rc[i] = r[i * rs];
    i64 front = 0, rear = 0;
    for (i64 i = 0; i < n; i++) {
        if (fabs(rc[i]) >= eps_vec[i]) {
            rear = (rear + 1) % (n + 2);
            queue[rear] = i;
            q_mark[i] = 1;
        }
    }
    i64 oper;
    if (!sor) {
        float *p = (float *)calloc((size_t)n, sizeof(float));
        oper = ign_push(n + 2, indptr, indices, degree, alpha, eps_vec, 1.0, 0, p, NULL, rc, queue, front, rear,
                        q_mark, beta);
        for (i64 i = 0; i < n; i++) p_out[i * ps] = (double)p[i];
        free(p);
    } else {
        double *p = (double *)calloc((size_t)n, sizeof(double));
        oper = ign_push(n + 2, indptr, indices, degree, alpha, eps_vec, omega, 1, NULL, p, rc, queue, front, rear,
                        q_mark, beta);
        for (i64 i = 0; i < n; i++) p_out[i * ps] = p[i];
        free(p);
    }
    for (i64 i = 0; i < n; i++) r[i * rs] = rc[i];
    free(eps_vec);
    free(rc);
    free(queue);
    free(q_mark);
    return oper;
}

/* updetaGraph (InstantGNN.py:137-180) == updeta_graph (ppr_solver.py:723-766).
 * Mutates indices/degree in place.  Outputs the insert/delete neighbour maps
 * in the reference's dict order: keys[] in first-insertion order, with
 * CSR-like offsets into nbr[].  Returns the number of insert keys; the delete
 * map is written to the d* arrays.  Arrays must hold 2*k entries. */
static i64 find_key(i64 *slot, i64 node) { return slot[node]; }

void orc_update_graph(i64 n, const i64 *indptr, i32 *indices, i64 *degree, const i64 *us, const i64 *vs, i64 k,
                      int onlyinsert, i64 *ins_keys, i64 *ins_off, i64 *ins_nbr, i64 *n_ins, i64 *del_keys,
                      i64 *del_off, i64 *del_nbr, i64 *n_del) {
    /* first gather per-key lists with insertion order, then flatten */
    i64 *ins_slot = (i64 *)malloc((size_t)n * sizeof(i64));
    i64 *del_slot = (i64 *)malloc((size_t)n * sizeof(i64));
    for (i64 i = 0; i < n; i++) ins_slot[i] = del_slot[i] = -1;
    i64 *ins_cnt = (i64 *)calloc((size_t)(2 * k + 1), sizeof(i64));
    i64 *del_cnt = (i64 *)calloc((size_t)(2 * k + 1), sizeof(i64));
    i64 *ev_key = (i64 *)malloc((size_t)(4 * k + 1) * sizeof(i64)); /* event log: key slot, neighbour */
    i64 *ev_nbr = (i64 *)malloc((size_t)(4 * k + 1) * sizeof(i64));
    int *ev_del = (int *)malloc((size_t)(4 * k + 1) * sizeof(int));
    i64 nev = 0, nik = 0, ndk = 0;
#define ADD_INS(a, b)                                     \
    do {                                                  \
        if (find_key(ins_slot, a) < 0) {                  \
            ins_slot[a] = nik;                            \
            ins_keys[nik++] = a;                          \
        }                                                 \
        ev_key[nev] = ins_slot[a];                        \
        ev_nbr[nev] = b;                                  \
        ev_del[nev++] = 0;                                \
        ins_cnt[ins_slot[a]]++;                           \
    } while (0)
#define ADD_DEL(a, b)                                     \
    do {                                                  \
        if (find_key(del_slot, a) < 0) {                  \
            del_slot[a] = ndk;                            \
            del_keys[ndk++] = a;                          \
        }                                                 \
        ev_key[nev] = del_slot[a];                        \
        ev_nbr[nev] = b;                                  \
        ev_del[nev++] = 1;                                \
        del_cnt[del_slot[a]]++;                           \
    } while (0)
    for (i64 e = 0; e < k; e++) {
        int insertion = 1;
        i64 u = us[e], v = vs[e];
        for (i64 i = indptr[u]; i < indptr[u] + degree[u]; i++) {
            if (v == indices[i]) {
                insertion = 0;
                if (onlyinsert || degree[u] == 1 || degree[v] == 1) break;
                indices[i] = indices[indptr[u] + degree[u] - 1];
                for (i64 kk = indptr[v]; kk < indptr[v] + degree[v]; kk++)
                    if (u == indices[kk]) indices[kk] = indices[indptr[v] + degree[v] - 1];
                degree[u] -= 1;
                degree[v] -= 1;
                ADD_DEL(u, v);
                ADD_DEL(v, u);
                break;
            }
        }
        if (insertion) {
            indices[indptr[u] + degree[u]] = (i32)v;
            indices[indptr[v] + degree[v]] = (i32)u;
            degree[u] += 1;
            degree[v] += 1;
            ADD_INS(u, v);
            ADD_INS(v, u);
        }
    }
#undef ADD_INS
#undef ADD_DEL
    ins_off[0] = 0;
    for (i64 i = 0; i < nik; i++) ins_off[i + 1] = ins_off[i] + ins_cnt[i];
    del_off[0] = 0;
    for (i64 i = 0; i < ndk; i++) del_off[i + 1] = del_off[i] + del_cnt[i];
    memset(ins_cnt, 0, (size_t)(2 * k + 1) * sizeof(i64));
    memset(del_cnt, 0, (size_t)(2 * k + 1) * sizeof(i64));
    for (i64 i = 0; i < nev; i++) {
        i64 sl = ev_key[i];
        if (ev_del[i]) del_nbr[del_off[sl] + del_cnt[sl]++] = ev_nbr[i];
        else ins_nbr[ins_off[sl] + ins_cnt[sl]++] = ev_nbr[i];
    }
    *n_ins = nik;
    *n_del = ndk;
    free(ins_slot);
    free(del_slot);
    free(ins_cnt);
    free(del_cnt);
    free(ev_key);
    free(ev_nbr);
    free(ev_del);
}

i64 orc_ign_sync_column(i64 n, const i64 *indptr, const i32 *indices, const i64 *degree, double alpha,
                        double x_gain, const double *eps_vec, double beta, double *p, double *r, i64 cs,
                        const unsigned char *cand0, i64 max_rounds);

/* instantGNNUpdateBatch for one column (InstantGNN.py:298-329).  p, r, x are
 * columns with stride cs; the maps are the outputs of orc_update_graph.
 * sync=1 keeps the reference's repair and replaces the FIFO push with the
 * synchronous push (candidates = the repaired nodes); sync=2 replaces it with
 * the multicolour SOR order given by color; both return the push's oper. */
i64 orc_ign_update_column(i64 n, const i64 *indptr, const i32 *indices, const i64 *degree, const i64 *old_degree,
                          double *p, double *r, const double *x, i64 cs, double alpha, double eps, double omega,
                          int sor, int insert_only, double beta, const i64 *ins_keys, const i64 *ins_off,
                          const i64 *ins_nbr, i64 n_ins, const i64 *del_keys, const i64 *del_off,
                          const i64 *del_nbr, i64 n_del, int sync, const i32 *color, i64 ncolors) {
    i64 sync_oper = 0;
    double *eps_vec = (double *)malloc((size_t)n * sizeof(double));
    double *pc = (double *)malloc((size_t)n * sizeof(double));
    double *rc = (double *)malloc((size_t)n * sizeof(double));
    i64 *queue = (i64 *)calloc((size_t)n + 2, sizeof(i64));
    unsigned char *q_mark = (unsigned char *)calloc((size_t)n, 1);
    i64 *del_slot = (i64 *)malloc((size_t)n * sizeof(i64));
    for (i64 i = 0; i < n; i++) del_slot[i] = -1;
    for (i64 i = 0; i < n_del; i++) del_slot[del_keys[i]] = i;
    for (i64 i = 0; i < n; i++) eps_vec[i] = pow((double)degree[i], 1 - beta) * eps;
    for (i64 i = 0; i < n; i++) { pc[i] = p[i * cs]; rc[i] = r[i * cs]; }
    for (i64 t = 0; t < n_ins; t++) {
        i64 u = ins_keys[t];
        double du = (double)degree[u], od = (double)old_degree[u];
        pc[u] *= pow(du / od, 1 - beta);
        rc[u] += pc[u] * (pow(od, 1 - beta) - pow(du, 1 - beta)) / pow(du, 1 - beta) * 1 / alpha;
    }
    i64 front = 0, rear = 0;
    for (i64 t = 0; t < n_ins; t++) {
        i64 u = ins_keys[t];
        double du = (double)degree[u], od = (double)old_degree[u];
        double dr = (pc[u] + alpha * rc[u] - alpha * x[u * cs]) * (pow(od, beta) - pow(du, beta)) / pow(du, beta);
        for (i64 q = ins_off[t]; q < ins_off[t + 1]; q++) {
            i64 v = ins_nbr[q];
            dr += (1 - alpha) * pc[v] / (pow(du, beta) * pow((double)degree[v], 1 - beta));
        }
        if (!insert_only && del_slot[u] >= 0) {
            i64 sl = del_slot[u];
            for (i64 q = del_off[sl]; q < del_off[sl + 1]; q++) {
                i64 v = del_nbr[q];
                dr -= (1 - alpha) * pc[v] / (pow(du, beta) * pow((double)degree[v], 1 - beta));
            }
        }
        rc[u] += dr / alpha;
        if (fabs(rc[u]) >= eps_vec[u]) {
            rear = (rear + 1) % (n + 2);
            queue[rear] = u;
            q_mark[u] = 1;
        }
    }
    if (sync) {
        unsigned char *cand0 = (unsigned char *)calloc((size_t)n, 1);
        for (i64 t = 0; t < n_ins; t++) cand0[ins_keys[t]] = 1;
        if (sync == 2)
            sync_oper = orc_ign_sor_color_column(n, indptr, indices, degree, alpha, eps_vec, beta, omega, pc, rc, 1,
                                                 cand0, color, ncolors, 0);
        else
            sync_oper = orc_ign_sync_column(n, indptr, indices, degree, alpha, alpha, eps_vec, beta, pc, rc, 1, cand0,
                                            (i64)1 << 40);
        free(cand0);
    } else if (rear != front) {
        ign_push(n + 2, indptr, indices, degree, alpha, eps_vec, omega, sor, NULL, pc, rc, queue, front, rear,
                 q_mark, beta);
    }
    for (i64 i = 0; i < n; i++) { p[i * cs] = pc[i]; r[i * cs] = rc[i]; }
    free(eps_vec);
    free(pc);
    free(rc);
    free(queue);
    free(q_mark);
    free(del_slot);
    return sync_oper;
}

/* update_ppr for one feature row (ppr_solver.py:769-821); sync as in orc_ign_update_column. */
i64 orc_update_ppr_row(i64 n, const i64 *indptr, const i32 *indices, const i64 *degree, const i64 *old_degree,
                       double *p, double *r, double alpha, double eps, double omega, const i64 *ins_keys,
                       const i64 *ins_off, const i64 *ins_nbr, i64 n_ins, const i64 *del_keys, const i64 *del_off,
                       const i64 *del_nbr, i64 n_del, int sync, const i32 *color, i64 ncolors) {
    double *eps_vec = (double *)malloc((size_t)n * sizeof(double));
    i64 *queue = (i64 *)calloc((size_t)n + 2, sizeof(i64));
    unsigned char *q_mark = (unsigned char *)calloc((size_t)n, 1);
    i64 *del_slot = (i64 *)malloc((size_t)n * sizeof(i64));
    for (i64 i = 0; i < n; i++) del_slot[i] = -1;
    for (i64 i = 0; i < n_del; i++) del_slot[del_keys[i]] = i;
    for (i64 i = 0; i < n; i++) eps_vec[i] = alpha * eps * (double)degree[i];
    i64 oper = 0, front = 0, rear = 0, qn = n + 2;
    oper += 2 * n_ins;
    for (i64 t = 0; t < n_ins; t++) {
        i64 u = ins_keys[t];
        p[u] *= (double)degree[u] / (double)old_degree[u];
        r[u] += p[u] * (double)(old_degree[u] - degree[u]) / (double)degree[u];
    }
    for (i64 t = 0; t < n_ins; t++) {
        i64 u = ins_keys[t];
        double dr = 0.;
        oper += ins_off[t + 1] - ins_off[t];
        for (i64 q = ins_off[t]; q < ins_off[t + 1]; q++) {
            i64 v = ins_nbr[q];
            dr += (1 - alpha) * p[v] / (double)degree[v];
        }
        if (del_slot[u] >= 0) {
            i64 sl = del_slot[u];
            oper += del_off[sl + 1] - del_off[sl];
            for (i64 q = del_off[sl]; q < del_off[sl + 1]; q++) {
                i64 v = del_nbr[q];
                dr -= (1 - alpha) * p[v] / (double)degree[v];
            }
        }
        r[u] += dr;
        if (fabs(r[u]) >= eps_vec[u]) {
            rear = (rear + 1) % qn;
            queue[rear] = u;
            q_mark[u] = 1;
        }
    }
    if (sync) {
        unsigned char *cand0 = (unsigned char *)calloc((size_t)n, 1);
        for (i64 t = 0; t < n_ins; t++) cand0[ins_keys[t]] = 1;
        if (sync == 2)
            oper += orc_ign_sor_color_column(n, indptr, indices, degree, alpha, eps_vec, 0.0, omega, p, r, 1, cand0,
                                             color, ncolors, 1);
        else
            oper += orc_ign_sync_column(n, indptr, indices, degree, alpha, 1.0, eps_vec, 0.0, p, r, 1, cand0,
                                        (i64)1 << 40);
        free(cand0);
        rear = front;  /* skip the FIFO push */
    }
    while (rear != front) {
        front = (front + 1) % qn;
        i64 u = queue[front];
        q_mark[u] = 0;
        if (fabs(r[u]) < eps_vec[u]) continue;
        if ((degree[u] == 1 && indices[indptr[u]] == u) || degree[u] == 0) {
            p[u] = r[u];
            r[u] = 0;
            continue;
        }
        double res_u = omega * r[u];
        p[u] += res_u;
        double push_u = (1. - alpha) * res_u / (double)degree[u];
        r[u] -= res_u;
        oper += degree[u];
        for (i64 e = indptr[u]; e < indptr[u] + degree[u]; e++) {
            i64 v = indices[e];
            r[v] += push_u;
            if (!q_mark[v] && fabs(r[v]) >= eps_vec[v]) {
                rear = (rear + 1) % qn;
                queue[rear] = v;
                q_mark[v] = 1;
            }
        }
        if (!q_mark[u] && fabs(r[u]) >= eps_vec[u]) {
            rear = (rear + 1) % qn;
            queue[rear] = u;
            q_mark[u] = 1;
        }
    }
    free(eps_vec);
    free(queue);
    free(q_mark);
    free(del_slot);
    return oper;
}

/* ------------------------------------------------------------------------ */
/* Synchronous InstantGNN push (the GPU's frontier rule), one column.        */
/* Rounds: F = {u in candidates : |r_u| >= eps_u}; absorbing nodes (degree 0 */
/* or a lone self-loop) move r into p; others p += a*r, r = 0, then push to  */
/* neighbours; candidates of the next round = nodes touched this round.      */
/* Returns the operation count sum over rounds of vol(F).                    */
/* ------------------------------------------------------------------------ */
i64 orc_ign_sync_column(i64 n, const i64 *indptr, const i32 *indices, const i64 *degree, double alpha,
                        double x_gain, const double *eps_vec, double beta, double *p, double *r, i64 cs,
                        const unsigned char *cand0, i64 max_rounds) {
    unsigned char *cand = (unsigned char *)malloc((size_t)n);
    unsigned char *next = (unsigned char *)calloc((size_t)n, 1);
    i64 *fr = (i64 *)malloc((size_t)n * sizeof(i64));
    double *val = (double *)malloc((size_t)n * sizeof(double));
    memcpy(cand, cand0, (size_t)n);
    i64 oper = 0;
    for (i64 round = 0; round < max_rounds; round++) {
        i64 nf = 0;
        for (i64 u = 0; u < n; u++)
            if (cand[u] && fabs(r[u * cs]) >= eps_vec[u]) fr[nf++] = u;
        if (nf == 0) break;
        memset(next, 0, (size_t)n);
        for (i64 i = 0; i < nf; i++) {
            i64 u = fr[i];
            double ru = r[u * cs];
            if ((degree[u] == 1 && indices[indptr[u]] == u) || degree[u] == 0) {
                p[u * cs] = ru;
                val[i] = 0.0;
            } else {
                p[u * cs] += x_gain * ru;
                val[i] = (1. - alpha) * ru / pow((double)degree[u], 1 - beta);
                oper += degree[u];
            }
            r[u * cs] = 0;
        }
        for (i64 i = 0; i < nf; i++) {
            i64 u = fr[i];
            if ((degree[u] == 1 && indices[indptr[u]] == u) || degree[u] == 0) continue;
            for (i64 e = indptr[u]; e < indptr[u] + degree[u]; e++) {
                i64 v = indices[e];
                r[v * cs] += val[i] / pow((double)degree[v], beta);
                next[v] = 1;
            }
        }
        unsigned char *t = cand;
        cand = next;
        next = t;
    }
    free(cand);
    free(next);
    free(fr);
    free(val);
    return oper;
}

/* ------------------------------------------------------------------------ */
/* Timed CPU baseline: many PPR local-GD queries, one query per thread.      */
/* x_out/r_out may be NULL (results discarded); oper_out[nq] receives opers. */
/* ------------------------------------------------------------------------ */
int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_ppr_gd_many(i64 n, const i64 *indptr, const i32 *indices, const double *degree, const i64 *seeds, i64 nq,
                     double alpha, const double *eps, int local, i64 *oper_out, double *x_out, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        double *x = (double *)malloc((size_t)n * sizeof(double));
        double *r = (double *)malloc((size_t)n * sizeof(double));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (i64 q = 0; q < nq; q++) {
            oper_out[q] = orc_ppr_gd(n, indptr, indices, degree, seeds[q], alpha, eps[q], local, x, r);
            if (x_out) memcpy(x_out + q * n, x, (size_t)n * sizeof(double));
        }
        free(x);
        free(r);
    }
}
