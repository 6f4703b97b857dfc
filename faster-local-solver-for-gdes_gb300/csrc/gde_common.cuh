// gde_common.cuh -- shared device/host definitions of the GB300 local push engine.
//
// The engine solves graph diffusion equations (PPR, Katz, heat kernel,
// InstantGNN feature propagation) by synchronous local push over a symmetric
// CSR graph.  Work is organised in *tiles*: a tile holds W solution columns
// (queries or feature columns) laid out node-major (element (u,c) at
// slab[u*ld + c]) so that one edge push moves W contiguous values with vector
// atomics, and the graph's column indices are read once per tile.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gde.h"

namespace gde {

// ---------------------------------------------------------------------------
// Problem kinds and methods (per tile)
// ---------------------------------------------------------------------------
enum Kind : int {
    KIND_PPR = 0,   // Q = I - (1-a) A D^-1, b = a e_s          (ppr_solver.py:18-23)
    KIND_KATZ = 1,  // Q = I - a A,          b = e_s            (katz_solver.py:177-179)
    KIND_HK = 2,    // Taylor-truncated heat kernel levels     (hk_solver.py:206-295)
    KIND_IGN = 3,   // generalised PPR with exponent beta      (InstantGNN.py:12-43)
    KIND_UPPR = 4,  // dynamic PPR update push, beta = 0 form  (ppr_solver.py:769-821)
};

enum Method : int {
    M_LOCAL_GD = 0,     // synchronous local push (LocalGD)
    M_GLOBAL_GD = 1,    // every node with r != 0 pushes each iteration
    M_LOCAL_CHEBY = 2,  // Chebyshev three-term recurrence on active nodes
    M_GLOBAL_CHEBY = 3,
    M_HK_LOCAL = 4,     // level-synchronous heat-kernel push (omega = 1)
    M_HK_GLOBAL = 5,    // every level sweeps all nodes
    M_HK_TAYLOR = 6,    // global Taylor series (hk_taylor_approx)
};

__host__ __device__ inline bool method_is_global(int m) {
    return m == M_GLOBAL_GD || m == M_GLOBAL_CHEBY || m == M_HK_GLOBAL || m == M_HK_TAYLOR;
}
__host__ __device__ inline bool method_is_cheby(int m) { return m == M_LOCAL_CHEBY || m == M_GLOBAL_CHEBY; }
__host__ __device__ inline bool method_is_hk(int m) { return m == M_HK_LOCAL || m == M_HK_GLOBAL || m == M_HK_TAYLOR; }

// ---------------------------------------------------------------------------
// Device graph
// ---------------------------------------------------------------------------
// Per-node record of a static graph: one 16-byte load gives a frontier
// node's row and degree.
struct __align__(16) NodeRec {
    long long rp;             // row start in col[]
    int len;                  // row length
    float degf;               // arithmetic degree
};

struct DevGraph {
    int64_t n;
    int64_t cap;              // capacity of col[] (nnz, or padded capacity)
    const int64_t* row_ptr;   // [n+2]; row u occupies col[row_ptr[u] .. row_ptr[u]+row_len[u])
    const int32_t* col;       // [cap]
    const int32_t* row_len;   // [n] live entries per row
    const float* degf;        // [n] arithmetic degree (exact for integer degrees < 2^24)
    const double* degd;       // [n] arithmetic degree in FP64
    const double* nfac;       // [n] InstantGNN threshold factor d^(1-beta) (nullptr otherwise)
    const double* npush;      // [n] InstantGNN push divisor d^(1-beta)
    const double* tfac;       // [n] InstantGNN target divisor d^beta
    const float* tfac_f;      // [n] same, FP32
    double vol;               // sum of degrees (m)
    int degf_exact;           // 1 when every degree is an integer < 2^24 (degf == degd exactly)
    const int32_t* perm;      // caller id -> internal id (nullptr: identity)
    int32_t hub_cut;          // internal ids < hub_cut are hubs (degree-sorted graphs; 0: none)
    // Static graphs with exact integer degrees: col_deg[j] = col[j] | code << idx_bits,
    // code = the target's degree, or deg_esc when it does not fit (read degf).
    // Lets a push test the target's threshold without a second random load.
    const uint32_t* col_deg;  // [cap] (nullptr: not built)
    int idx_bits;
    uint32_t deg_esc;
    const NodeRec* rec;       // [n] (nullptr: not built)
};

// ---------------------------------------------------------------------------
// Per-tile state
// ---------------------------------------------------------------------------
constexpr int kMaxW = 32;

struct TileParams {           // host-written, read-only during a launch
    int kind, method;
    int ncols;                // live column slots (<= W)
    int n_levels;             // HK: N (levels 0..N-1), Taylor: N (levels 0..N)
    double alpha, tau;
    double l_max, mu_min;     // Katz Chebyshev spectral bounds
    double beta;              // InstantGNN exponent
    double x_gain;            // InstantGNN: p += x_gain * r (alpha); dynamic PPR: 1
    const double* coef_tab;   // Chebyshev: beta_t (PPR) or (beta1_t, beta2_t) pairs (Katz), per round
    const double* psi_tab;    // HK: psi[0..N]
    int64_t seed_base;        // unused by the kernel (bookkeeping)
    double omega;             // HK: relaxation of hk_sor_queue (0 and 1: none)
};

// HK relaxation omega != 1 (hk_solver.py:248-264): each push moves omega r
// and keeps (1 - omega) r at its level.
__host__ __device__ inline bool hk_relaxed(const TileParams& tp) { return tp.omega != 0.0 && tp.omega != 1.0; }
constexpr int kMaxRelax = 1 << 16;  // bound on the sub-pushes of one node at one level

// Counter discipline (no phase ever reads a field another block writes in
// the same phase).  Round r of a tile has level = ts.round + it, parity
// p = level & 1:
//   PREP(r)    reads cand_cnt[r%3]; writes front/small/med/large/union_vol[p],
//              round_active[p]; appends (Chebyshev) to cand_cnt[(r+1)%3];
//              block 0 zeroes the p^1 counters and cand_cnt[(r+2)%3].
//   SCATTER(r) reads the p counters; appends to cand_cnt[(r+1)%3]; block 0
//              writes ts.done / dense_next[p^1] / ColState.live, which are
//              only read at the start of the next round.
enum SlotState : int {
    SLOT_LIVE = 0,    // pushing; level = it - t0
    SLOT_DONE = 1,    // finished (batch solves: results extracted after the launch)
    SLOT_IDLE = 2,    // served solves: result extracted and slot cleared, awaiting a query
    SLOT_EMPTY = 3,   // served solves: no query left for this slot
    SLOT_DRAIN = 4,   // online server: result written; the slot's vectors are cleared this round
};

// ---------------------------------------------------------------------------
// Online server (gde_server_*): requests arrive in a ring in pinned host
// memory that the device reads while the persistent launch runs.
// ---------------------------------------------------------------------------
struct OnlineReq {            // one submitted query, written by the host before it publishes `tail`
    int32_t kind;             // KIND_PPR / KIND_KATZ / KIND_HK
    int32_t seed;             // internal node id
    int32_t seed_caller;      // caller node id (Katz x[s] -= 1 in caller order)
    int32_t n_levels;         // HK: Taylor length N
    int32_t psi_off;          // HK: offset of its psi table
    int32_t out64;            // x_out holds doubles (else floats)
    double theta;             // threshold scale
    double r0;                // initial residual at the seed
    double alpha;             // PPR / Katz alpha
    void* x_out;              // device-addressable row of n entries, caller order (nullptr: none)
    long long ticket;
};

struct OnlineDone {           // completion record, device-written; the host reads done_ticket last
    double oper;
    int32_t rounds;
    int32_t status;           // GDE_OK
    unsigned long long admit_ns, finish_ns;
    long long done_ticket;    // == ticket once the record and the row are complete
};

struct OnlineSlot {           // the query a slot holds (copied out of the ring at admission)
    long long ticket;
    void* x_out;
    int32_t out64;
    int32_t seed_caller;
    int32_t kind;
    int32_t rounds;
    int32_t status;           // GDE_OK, or GDE_EITERCAP when max_rounds stopped it
    int32_t pending;          // 1: `mail` holds a request for this idle slot, not admitted yet
    double oper;
    unsigned long long admit_ns, finish_ns;
    OnlineReq mail;           // written by the ring reader, read by the slot's own group at admission
};

struct TileState {            // device-updated
    int cand_cnt[3];          // candidate list sizes (by level mod 3)
    int front_cnt[2];         // frontier sizes (by parity)
    int small_cnt[2], med_cnt[2], large_cnt[2];
    int dense_next[2];        // 1: the PREP of that parity scans all nodes
    int t0;                   // launch iteration at which the tile's level 0 ran
    int done;                 // SlotState
    int stamp;                // touch-stamp base (marks start at -1; stamps only grow)
    int qid;                  // served solves: query in this slot (-1 none)
    double union_vol[2];      // volume of the union frontier per round parity
};

// Served solves: a queue of single-column queries cycling through the slots.
struct ServeQueue {
    int nq;                       // queries in the queue
    int* next;                    // next query to admit (device counter)
    const int32_t* seed;          // internal seed id per query
    const double* theta;          // threshold scale per query
    const double* r0;             // initial residual at the seed
    const long long* arrival_ns;  // admission not before kernel start + arrival (nullptr: immediately)
    void* x_out;                  // [nq][ld_out] solution rows, caller node order
    void* r_out;                  // [nq][ld_out] residual rows (may be null)
    int64_t ld_out;
    int out64;
    double seed_add;              // single-kind queues (kind == nullptr): added to x[seed]
    // mixed queues (nullptr: every query is of the launch's tile kind)
    const int32_t* kind;          // KIND_PPR / KIND_KATZ / KIND_HK per query
    const double* alpha;          // PPR / Katz alpha per query
    const int32_t* n_levels;      // HK: Taylor length N per query
    const int32_t* psi_off;       // HK: offset of the query's psi table in psi
    const double* psi;            // HK: psi tables, concatenated
    double tau;                   // HK temperature
    double hk_scale;              // HK: x is divided by e^tau
    double* oper;                 // [nq] operation counts
    int* rounds;                  // [nq]
    unsigned long long* start_ns; // [nq] admission time
    unsigned long long* finish_ns;// [nq] finish time
    // online server (online != 0): queries come from a ring the host fills
    // while the launch runs, instead of the arrays above
    int online;
    int cap;                      // ring entries
    const OnlineReq* req;         // [cap] pinned host ring
    OnlineDone* done;             // [cap] pinned host completion records (ticket % cap)
    const long long* tail;        // host-written: tickets submitted so far
    long long* head;              // device-written (host-visible): tickets admitted so far
    const int* stop;              // host-written stop flag
    int* quit;                    // device: set by the ring reader (stop flag, or idle) for every group
    int* gquit;                   // device [groups]: each group's copy of quit, taken before its round's
                                  // last barrier, so that all its blocks leave at the same round start
    unsigned long long* last_ns;  // device: %globaltimer of the last round with work
    unsigned long long idle_ns;   // the launch ends after this long with nothing to do
    OnlineSlot* slot;             // [slots]
    const int32_t* perm;          // caller id -> internal id (nullptr: identity)
    // Hash-compacted small queries (sp_blocks > 0): the launch's last
    // sp_blocks blocks each solve one PPR / Katz local GD query at a time
    // out of an open-addressing table of sp_cap entries in global memory
    // (keys, FP64 residual and solution), instead of dense vectors.  Queries
    // in order_s go there; one whose touched set outgrows the table is queued
    // for the dense slots (ovf).  Dense slots take order_d (nullptr: query
    // ids in order), then the overflow list.  A finished sparse query writes
    // its entries into its {x, c} query slab (the launch needs xq != 0), so
    // the read-out after the launch is the same for both classes.
    int sp_blocks;
    int sp_cap;                   // entries per table (power of two)
    const int32_t* order_d;       // [nd] dense-class query ids, in arrival order
    int nd;
    const int32_t* order_s;       // [ns] sparse-class query ids, in arrival order
    int ns;
    int* next_s;                  // next order_s position
    int* ovf;                     // [ns] overflowed query ids, -1 until written
    int* ovf_cnt;                 // ovf positions handed out
    int* ovf_next;                // next ovf entry to admit
    int* sp_left;                 // sparse-class queries not yet finished or overflowed
    int32_t* sp_keys;             // [sp_blocks][sp_cap] node id per entry (-1: empty)
    double* sp_r;                 // [sp_blocks][sp_cap] residual
    double* sp_x;                 // [sp_blocks][sp_cap] solution
    int32_t* sp_list;             // [sp_blocks][3][sp_cap] frontier (two) and used-entry lists
    double* sp_push;              // [sp_blocks][sp_cap] push value per frontier entry
    int kind0;                    // single-kind queues: the queries' kind
    double alpha0;                //                     and alpha
};

struct ColState {             // one per column slot
    double theta;             // threshold scale (eps*alpha, eps, e^tau*eps, eps ...)
    double oper;              // operation count (sum of degrees of pushed nodes)
    int64_t fsum;             // sum over rounds of frontier size
    int live;                 // 1 while the column still has active nodes
    int rounds;               // rounds in which the column pushed
    int round_active[2];      // active nodes this round (parity)
    int check_cnt[2];         // global methods: nodes above threshold (parity)
    int seed;                 // seed node (-1 for feature columns)
    int pad;
    int hk_sweeps[2];         // HK global sweeps, omega != 1: sweeps of the level (parity), max over nodes
    int64_t sweep_sum;        // HK global sweeps, omega != 1: sweeps over all levels
    unsigned long long finish_ns;  // %globaltimer when the column finished (0 = not yet)
};

struct LaunchStats {          // roofline counters summed over a launch
    unsigned long long union_nodes;    // sum_t |U S_t| (per tile)
    double union_vol;                  // sum_t vol(U S_t)
    unsigned long long col_nodes;      // sum_t sum_c |S_t^c|
    double col_vol;                    // sum_t sum_c vol(S_t^c)
    unsigned long long dense_rounds;
    unsigned long long rounds;
    unsigned long long cand_nodes;     // candidates examined
    unsigned long long start_ns;       // %globaltimer at kernel start (block 0)
    unsigned long long check_ns;       // block 0's time in CHECK phases (incl. barrier wait)
    unsigned long long prep_ns;        // ... PREP phases
    unsigned long long scatter_ns;     // ... SCATTER phases
    unsigned long long iters;          // launch iterations run
    unsigned long long sp_done;        // served small queries finished in hash tables
    unsigned long long sp_ovf;         // ... handed to the dense slots
};

// Arrival counter and generation word on separate 128-byte lines: waiting
// blocks poll `gen` without slowing the arrivals on `count`.
struct GridBarrier {
    unsigned int count;
    unsigned int pad0[31];
    unsigned int gen;
    unsigned int pad1[31];
};

// A piece of push work: `len` edges of one frontier row starting at col[rp]
// (a whole short/medium row, or one chunk of a long row), and the row's
// frontier index (its push values are P[fidx][0..W)).
struct PushItem {
    long long rp;
    int len;
    int fidx;
};

// Engine launch parameters (passed by value to the persistent kernel).
struct PushArgs {
    DevGraph g;
    int ntiles;
    int ld;                    // row stride of the slabs (elements)
    int64_t tile_stride;       // element offset between consecutive tiles' slabs
    void* R;                   // residual slab (levels 0,2,4.. for HK)
    void* R2;                  // HK odd-level residual slab
    void* X;                   // solution slab
    float* XC;                 // Kahan compensation (FP32 solution), may be null
    int xld;                   // X / XC row stride; 0: the slabs' ld.  2 = interleaved
                               // {x, c} pairs (W = 1 Kahan slabs: XC = (float*)X + 1)
    int64_t xtile;             // X / XC offset between tiles (with xld != 0)
    int xq;                    // served: X / XC slabs per query (indexed by query id), read out
                               // after the launch; 0: per tile
    void* DX;                  // Chebyshev delta-x slab
    int32_t* cand;             // [ntiles][2][n] (list storage by parity)
    void* P;                   // [ntiles][n][W] push rows
    PushItem* bsmall;          // [ntiles][n]   short rows from index 0 up, medium rows from n-1 down
    PushItem* blarge;          // [ntiles][large_cap]  chunks of long rows
    int64_t large_cap;
    int32_t* mark;             // [ntiles][n]
    TileParams* tp;            // [ntiles]
    TileState* ts;             // [ntiles]
    ColState* cs;              // [ntiles][W]
    LaunchStats* stats;
    GridBarrier* bar;
    int* err;
    int small_max;             // rows with len <= small_max: lane group per row
    int med_max;               // rows with len <= med_max: warp per row; else CTA chunks
    int chunk;                 // edges per CTA chunk (large rows)
    int dense_div;             // frontier volume > n/dense_div -> next round scans densely
    int max_rounds;            // hard cap on a tile's rounds
    int round_budget;          // rounds to advance in this launch (serving ticks)
    int kahan;                 // compensated FP32 solution
    int allow_dense;           // 0: every round visits only touched nodes (dynamic updates)
    int serve;                 // 1: slots (W = 1 tiles) cycle through `queue`
    ServeQueue queue;
    unsigned long long* trace; // [trace_iters][grid][kTracePoints] %globaltimer stamps (nullptr: off)
    int trace_iters;
    unsigned long long spin_limit;  // grid-barrier polls before GDE_EHANG (0: the default, ~seconds)
    // Served solves: the grid splits into `groups` block groups (blocks
    // [g B / G, (g+1) B / G)), each advancing the slots t with t % G == g
    // behind its own barrier bar[g], so a straggler stalls only its group.
    // 0 or 1: one group (every other launch).
    int groups;
    // Served one-column FP32 slots of PPR / Katz local GD: the residual of the
    // highest-degree nodes (internal ids < rh_cut of a degree-sorted graph)
    // accumulates in FP64, rh_cut entries per slot.  Those nodes take
    // thousands of additions per round, and one threshold flip there moves
    // about 2 theta d of l1.  nullptr: every residual entry is in R.
    double* RH;
    int rh_cut;
};

constexpr int kMaxGroups = 512;  // at most one per slot (kMaxLaunchTiles)

// Phase boundaries stamped per block and launch iteration when tracing is on.
enum TracePoint : int {
    TP_ITER = 0,        // iteration start
    TP_PREP_WORK,       // after the round set-up, PREP work begins
    TP_PREP_DONE,       // PREP work done, entering the grid barrier
    TP_PREP_BAR,        // PREP barrier passed
    TP_SCAT_WORK,       // SCATTER set-up (scans, retire) done, push work begins
    TP_SCAT_DONE,       // push work done (before HK drop / block-0 bookkeeping)
    TP_SCAT_ENTER,      // entering the SCATTER grid barrier
    TP_SCAT_BAR,        // SCATTER barrier passed
    kTracePoints
};

}  // namespace gde
