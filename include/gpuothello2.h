/*
 * gpuothello2.h -- C ABI of the GB300 batched exact Othello endgame solver.
 *
 * The reference drives its GPU solver through a C++ class, BatchedTask
 * (solver.cuh:8-25; solver.cu:313-348): construct with (batch_size,
 * max_depth, Table&), fill `abp[]` = AlphaBetaProblem{player, opponent}
 * (alphabeta.cuh:13-21) in managed memory, launch(), poll is_ready(), read
 * `result[]` (int32) -- with the CLI's solve() doing exactly that
 * (main.cu:123-173).  This header replaces that class with plain functions
 * over caller-owned host (or device) arrays, so any language with a C FFI can
 * bind it.
 *
 * Conventions
 *   - A position is two disjoint 64-bit bitboards: `player` = discs of the
 *     side to move, `opp` = discs of the other side; square = row*8 + col,
 *     A1 = bit 0 (main.cu:31-39).
 *   - Scores are exact final disc differences from the side to move, with
 *     the empty squares awarded to the winner (board.cuh:7-18): even
 *     integers in [-64, 64].
 *   - `depth` is the reference's DEPTH: the largest number of empty squares
 *     any position of the batch may have (README.md:56-58).  A position with
 *     more empties than `depth` is an error, not undefined behaviour.
 *   - All calls are synchronous and serialised by an internal lock.  Device
 *     buffers, the stream and the transposition table live in one library
 *     context per CUDA device, created on first use on the device current at
 *     the call (so a caller may switch devices between calls) and released by
 *     solve_shutdown().  The learned orderer's network lives on the device
 *     current at gpo_mlp_load; solves on other devices run without it.
 *   - Every entry point returns GPO_OK (0) or a negative GPO_ERR_* status.
 */
#ifndef GPUOTHELLO2_H
#define GPUOTHELLO2_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPO_OK 0
#define GPO_ERR_ARG (-1)      /* null pointer, n < 0, bad option value */
#define GPO_ERR_DEPTH (-2)    /* depth out of [1, 32] or a position has more empties than depth */
#define GPO_ERR_BOARD (-3)    /* a square is set in both bitboards */
#define GPO_ERR_CUDA (-4)     /* CUDA runtime error (no device, launch failure, ...) */
#define GPO_ERR_NOMEM (-5)    /* device or pinned-host allocation failed */
#define GPO_ERR_TIMEOUT (-6)  /* node_budget exceeded, or the search passed wait_limit_ms */
#define GPO_ERR_INTERNAL (-7) /* a kernel consistency check failed */
#define GPO_ERR_IO (-8)       /* file could not be read or written */

/* Move codes in best-move outputs: 0..63 = square, 64 = pass, 65 = no move
 * (game over) -- the reference's hand::PASS / hand::NOMOVE (alphabeta.cuh:7-10). */
#define GPO_MOVE_PASS 64
#define GPO_MOVE_NONE 65

/* Search methods. */
#define GPO_METHOD_BATCHED 0 /* persistent, empties-bucketed kernel (default) */
#define GPO_METHOD_PLAIN 1   /* thread-per-board kernel, the reference's exact tree */

typedef struct gpo_options {
  int method;                 /* GPO_METHOD_* */
  int use_table;              /* transposition table: 0 off, 1 or -1 (auto) on; cleared at
                                 every call, so no result carries over */
  int use_learned;            /* learned move ordering (gpo_mlp_load): -1 auto (on when a
                                 network is loaded on this device), 0 off, 1 on */
  int threads_per_block;      /* 32..256, multiple of 32; 0 = 128 */
  int fastest_first_empties;  /* fastest-first ordering at nodes with >= this many empties;
                                 0 = default (6) */
  int learned_min_empties;    /* learned ordering at the nodes with >= this many empties in
                                 the top two plies of each position; 0 = 12 */
  uint64_t node_budget;       /* per-position node limit, 0 = none (watchdog: GPO_ERR_TIMEOUT) */
  int help_min_empties;       /* idle lanes of a warp help its busy lanes with moves of nodes
                                 that have >= this many empties (young brothers wait, after
                                 the node's first move); 0 = default (7), negative = off */
  int wait_limit_ms;          /* deadline of one search launch; 0 = 600000 */
  int table_bits;             /* transposition table of 2^table_bits 16-byte entries in
                                 buckets of two (17..32); 0 = 28 (4 GiB) on a device with
                                 >= 64 GiB of memory, else 24 (256 MiB) */
  int table_min_empties;      /* nodes with >= this many empties use the table; 0 = 9 */
  int smem_frames;            /* search frames (depth - 2 slots per lane) in shared memory:
                                 0 = when they all fit at the register-limited occupancy,
                                 > 0 = only if at most this many are needed, negative = never
                                 (every frame in the global frame array) */
  int stability_min_empties;  /* stability cutoff at nodes with >= this many empties (and
                                 alpha >= 10 + 3 * empties); 0 = default (4), negative = off */
  int roots_per_warp;         /* input positions a warp searches at once, the rest of its
                                 lanes helping (1..32); 0 = from the batch size: 32 when the
                                 batch fills the GPU, fewer for small batches */
  int64_t hard_nodes;         /* a warp whose own search has visited more than this many
                                 nodes takes no new positions, so its lanes help that search
                                 as they come free; 0 = default (2^23), negative = off */
  int root_split_plies;       /* batches with fewer positions than 1/8 of the GPU's warps
                                 (depth >= 14): 0 = expanded on the host until the frontier
                                 fills the GPU (at most 3 plies; positions with <= 12 empties
                                 are not expanded), every frontier position solved exactly in
                                 one launch, values taken back up by negamax; > 0 = always
                                 expand this many plies; negative = never */
  int tail_split_positions;   /* tail handoff (depth >= 14): once every position has been
                                 taken up and at most this many are unfinished, their
                                 searches stop and a root split finishes them over the whole
                                 GPU, the table kept and the frontier searched with windows
                                 from what the stopped searches proved; 0 = default (1/16 of
                                 the GPU's warps), negative = off */
} gpo_options;

typedef struct gpo_stats {
  uint64_t nodes;          /* positions visited (root, children, pass frames; with a tail
                              handoff, the stopped searches' nodes too) */
  uint64_t table_probes;   /* transposition-table lookups */
  uint64_t table_hits;     /* lookups that found the position */
  uint64_t table_updates;  /* stores into the table */
  uint64_t learned_calls;  /* positions scored by the learned orderer */
  uint64_t splits;         /* moves of split nodes searched by helper lanes */
  double kernel_ms;        /* device time of the search kernel (CUDA events; with a root
                              split or a tail handoff, of every search launch) */
  double total_ms;         /* wall time of the call */
  uint64_t launches;       /* kernels the call launched */
  uint64_t stability_cuts; /* nodes closed by the stability cutoff */
  uint64_t table_bits;     /* log2 of the table's entries used by the call (0 = no table) */
  uint64_t root_split_positions; /* frontier positions a root split solved (0 = no split) */
  uint64_t tail_positions; /* positions finished by the tail handoff's root split */
} gpo_stats;

/* Fills *opt with the defaults (all fields "auto"/0). */
void gpo_default_options(gpo_options* opt);

/*
 * Exact-solves n positions.  player/opp/score are caller-owned host arrays
 * of n elements; score[i] receives the exact score of position i.
 * Replaces BatchedTask ctor + abp fill + launch + is_ready polling + result
 * read-back (solver.cuh:8-25, solver.cu:313-348, main.cu:135-171).
 */
int solve_batch(const uint64_t* player, const uint64_t* opp, int n, int depth, int8_t* score);

/*
 * As solve_batch, with options (NULL = defaults), an optional best-move
 * output (NULL = not wanted; 0..63, GPO_MOVE_PASS or GPO_MOVE_NONE), an
 * optional per-position node count output (NULL = not wanted) and optional
 * statistics (NULL = not wanted).  The table counters of gpo_stats are the
 * reference's "table update count / hit / find" (table.cuh:26-40,
 * main.cu:158-162).
 */
int solve_batch_ex(const uint64_t* player, const uint64_t* opp, int n, int depth, int8_t* score,
                   int8_t* best_move, uint64_t* nodes, const gpo_options* opt, gpo_stats* stats);

/*
 * As solve_batch_ex, but every array is a device pointer on the current
 * device and the work is ordered on `stream` (a cudaStream_t; NULL = the
 * library's own stream).  Returns after the work completes.
 */
int solve_batch_device(const uint64_t* d_player, const uint64_t* d_opp, int n, int depth,
                       int8_t* d_score, int8_t* d_best_move, uint64_t* d_nodes,
                       const gpo_options* opt, gpo_stats* stats, void* stream);

/*
 * Generates n positions of the seeded random-playout stream `seed`, indices
 * first .. first+n-1, on the GPU (host output arrays).  Empty count is
 * min_empties when min == max, else uniform in [min_empties, max_empties].
 * Definition: xoshiro256** seeded with four successive splitmix64 outputs
 * from x0 = (seed << 32) + index; uniform(k) = high 64 bits of next() * k;
 * the empty count (if ranged) is drawn first; from the standard start
 * (black to move, black d5/e4, white d4/e5) play the uniform(k)-th set bit
 * of the k legal moves (from bit 0), pass when only the other side can move,
 * restart the game (same PRNG stream) if it ends early, and stop when exactly
 * the wanted number of squares is empty.
 */
int gpo_generate(uint64_t seed, uint64_t first, int n, int min_empties, int max_empties,
                 uint64_t* player, uint64_t* opp);
int gpo_generate_device(uint64_t seed, uint64_t first, int n, int min_empties, int max_empties,
                        uint64_t* d_player, uint64_t* d_opp, void* stream);

/*
 * Repeated batches as a CUDA graph.  The reference launches one BatchedTask
 * per batch on its own stream and polls it (main.cu:146-155,
 * solver.cu:330-333); a caller that solves batch after batch of the same
 * size in the same device arrays can instead capture the batched solve once
 * and replay it.  gpo_graph_create captures the solve of n positions held in
 * d_player/d_opp (scores to d_score) with the given options (NULL =
 * defaults; the learned ordering, the root split of small batches and the
 * tail handoff need host decisions and are left out: use_learned must not be
 * 1); the graph owns
 * its scratch and table.  gpo_graph_launch replays it on `stream` (NULL =
 * the legacy default stream) and returns at once: refill the inputs in place
 * between replays, ordered on the same stream.  gpo_graph_stats, after the
 * stream has finished, gives the last replay's counters and status
 * (GPO_ERR_* for rejected inputs or an exceeded deadline).  A graph is bound
 * to the device current at its creation.
 */
typedef struct gpo_graph gpo_graph;
int gpo_graph_create(const uint64_t* d_player, const uint64_t* d_opp, int n, int depth,
                     int8_t* d_score, const gpo_options* opt, gpo_graph** graph);
int gpo_graph_launch(gpo_graph* graph, void* stream);
int gpo_graph_stats(gpo_graph* graph, gpo_stats* stats);
void gpo_graph_destroy(gpo_graph* graph);

/*
 * No counterpart in the reference.  The batched solver for callers that
 * cannot allocate device memory (a host program whose pool allocator owns
 * all device memory, a plugin that may not allocate after start-up, code that
 * must avoid the device synchronisation an allocation can cause).  It
 * allocates nothing: its scratch lives in a fixed array inside the library
 * (about 12 MiB, held by every GPU that loads the library until exit).
 * Device input and score arrays as in solve_batch_device; `stream` may be
 * NULL (the legacy default stream).  At most GPO_NOALLOC_MAX_POSITIONS
 * positions (else GPO_ERR_ARG) and depth <= GPO_NOALLOC_MAX_DEPTH (else
 * GPO_ERR_DEPTH).  The transposition table and the learned ordering are off;
 * the lanes of a warp help each other as in solve_batch_device.  When the
 * frame slots do not fit in shared memory and would not fit the array for the
 * full grid, the launch uses the largest grid that fits.  The first call on a
 * device looks up the array's address; make it before any stream capture.
 * The call returns after its work on `stream` has finished.  Calls share the
 * array: calls that overlap on the GPU race.
 */
#define GPO_NOALLOC_MAX_POSITIONS (1 << 20)
#define GPO_NOALLOC_MAX_DEPTH 16
int solve_batch_device_noalloc(const uint64_t* d_player, const uint64_t* d_opp, int n, int depth,
                               int8_t* d_score, void* stream);

/*
 * Learned move orderer (no counterpart in the reference).  An MLP 192 -> 256 -> 256 -> 64 over (side-to-move discs,
 * other discs, legal moves) with BF16 tensor-core products and FP32
 * accumulation, trained on the GPU on best-move labels from
 * solve_batch_ex.  Weights are a flat FP32 array of gpo_mlp_param_count()
 * values: W1[192][256], b1[256], W2[256][256], b2[256], W3[256][64], b3[64].
 * gpo_mlp_load makes the solver order the moves of the nodes with
 * >= learned_min_empties empties in the top two plies of each position by
 * the network (scores stay exact); the nodes are scored in large batches
 * before the search.  The network is loaded on the current device (NULL
 * unloads it); a reload waits for inference already enqueued by a solve.
 */
int gpo_mlp_param_count(void);
int gpo_mlp_init(uint64_t seed, float* weights);
int gpo_mlp_forward(const float* weights, const uint64_t* player, const uint64_t* opp, int n,
                    float* logits);
int gpo_mlp_gradients(const float* weights, const uint64_t* player, const uint64_t* opp,
                      const int8_t* best, int n, float* grads, float* loss);
int gpo_mlp_train(const uint64_t* player, const uint64_t* opp, const int8_t* best, int n,
                  int epochs, int batch, float lr, uint64_t seed, float* weights, float* history);
int gpo_mlp_load(const float* weights);

/*
 * Think mode: depth-limited search with a pattern evaluator, the reference's
 * `solver INPUT OUTPUT DEPTH THINK_DEPTH` path (main.cu:69-121).
 *
 * gpo_eval_load replaces Evaluator's constructor (eval.cu:12-60):
 * features[n_features] are square masks (at most 32 features of at most 12
 * squares each); values holds every feature's table in order (3^k doubles
 * for a k-square feature, indexed by the base-3 number whose digit j is 0
 * empty, 1 side to move, 2 other side on the mask's j-th lowest square),
 * stored as float like the reference; offset is added to the sum.
 * gpo_eval_load_files reads the same from the reference's feature file
 * (count, then 8 rows of 8 binary digits per feature) and value file
 * (binary doubles, then the offset); GPO_ERR_IO if a file is missing or
 * short, GPO_ERR_ARG if malformed.
 */
int gpo_eval_load(const uint64_t* features, int n_features, const double* values, double offset);
int gpo_eval_load_files(const char* features_path, const char* values_path);
/* Evaluator::eval (eval.cu:129-141) of n positions: the sum over the 8
 * board symmetries and all features, plus the offset, clamped to [-64, 64].
 * GPO_ERR_ARG if no evaluator is loaded. */
int gpo_evaluate(const uint64_t* player, const uint64_t* opp, int n, float* value);
/* Replaces BatchedThinkTask + think_kernel (thinker.cuh:9-29,
 * thinker.cu:12-389): searches each position `depth` plies (4..24; passes
 * take none) and scores the positions reached with round(eval); games that
 * end earlier are scored exactly.  score[i] = the value for the side to
 * move; best_move[i] (optional) = its move, 64 = pass; nodes[i] (optional)
 * = positions visited (root, children, pass frames, leaves).  Any number of
 * empty squares.  GPO_ERR_ARG if no evaluator is loaded, GPO_ERR_DEPTH for
 * a depth outside 4..24, GPO_ERR_BOARD for overlapping bitboards. */
int think_batch(const uint64_t* player, const uint64_t* opp, int n, int depth, int8_t* score,
                int8_t* best_move, uint64_t* nodes, gpo_stats* stats);

/* Releases the library context (device buffers, table, stream). */
void solve_shutdown(void);

/* Human-readable text for a status code. */
const char* gpo_strerror(int status);

/* Name of the device the context runs on, and its SM count (0 if none). */
int gpo_device_info(char* name, int name_len, int* sm_count);

#ifdef __cplusplus
}
#endif
#endif /* GPUOTHELLO2_H */
