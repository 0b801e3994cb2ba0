/*
 * CPU oracle for the batched exact endgame solver -- TEST INFRASTRUCTURE.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library, and only as the checker or the timed CPU baseline; the
 * product (libgpuothello2.so, the `solver` CLI) never links or calls it.
 *
 * It restates, in plain C, the reference's algorithm for the solve path:
 *   - bitboard flip / mobility / final score   (board.cu:28-86, board.cuh:7-18)
 *   - the reference's exact search tree: upper plies ordered by opponent
 *     mobility, lower plies corners-first then lowest square, fail-soft
 *     negamax with pass handling (solver.cu:75-283, node.cuh:5-74)
 *   - the base81 board codec (test.cpp:7-19 encoder, to_board.cpp:15-39
 *     decoder semantics)
 *   - the pattern evaluator and the depth-limited think-mode search
 *     (eval.cu:12-141, thinker.cu:12-376)
 * plus an independent fast alpha-beta solver (different move ordering, so
 * a second opinion on every score) and the seeded random-playout position
 * generator that defines the benchmark inputs.
 *
 * Parity is pinned against the reference itself: tests/golden/ holds scores
 * and per-position loop-step counts produced by the reference's own search
 * code (oracle/ref_build.sh) and the oracle must reproduce both exactly.
 */
#ifndef GPO_ORACLE_H
#define GPO_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- bitboards: square = row*8 + col, A1 = bit 0 (main.cu:31-39) ---- */
uint64_t orc_flip(uint64_t p, uint64_t o, int sq);
uint64_t orc_flip_naive(uint64_t p, uint64_t o, int sq);
uint64_t orc_mobility(uint64_t p, uint64_t o);
uint64_t orc_mobility_naive(uint64_t p, uint64_t o);
int orc_final_score(uint64_t p, uint64_t o);

/* ---- base81 codec: 16 chars per board ---- */
void orc_encode(uint64_t p, uint64_t o, char out[17]);
/* Returns 0 on success, -1 if a char is outside the codec's alphabet or a
 * square is claimed by both sides. */
int orc_decode(const char* s, uint64_t* p, uint64_t* o);

/* ---- seeded random-playout generator ---- */
/* Position i of stream `seed` (i = first_index .. first_index+n-1).  Empty
 * count is min_empties when min == max, else drawn uniformly from
 * [min_empties, max_empties] first.  See orc_generate in oracle.c for the
 * exact PRNG definition. */
void orc_generate(uint64_t seed, uint64_t first_index, int n, int min_empties,
                  int max_empties, uint64_t* p, uint64_t* o);

/* ---- solvers ---- */
/* Reference-order search.  Returns the exact score (side to move); *steps
 * receives the reference's loop-step count (solver.cu:273-275) and *nodes
 * the number of positions pushed (root, children and pass frames).
 * depth must be >= 10 and >= the empty count (solver.cu:9, 322). */
int orc_solve_ref(uint64_t p, uint64_t o, int depth, uint64_t* steps, uint64_t* nodes);
/* Independent alpha-beta (fastest-first + parity ordering).  Returns the
 * exact score; *best receives a move achieving it (64 = pass, 65 = none). */
int orc_solve_fast(uint64_t p, uint64_t o, uint64_t* nodes, int* best);
/* Multithreaded batch: mode 0 = reference order, 1 = fast.  steps/nodes/best
 * may be NULL.  threads <= 0 means all online cores.  Returns 0. */
int orc_solve_batch(const uint64_t* p, const uint64_t* o, int n, int depth, int mode,
                    int threads, int8_t* score, uint64_t* steps, uint64_t* nodes, int8_t* best);
int orc_num_cores(void);

/* ---- pattern evaluator and think mode (eval.cu, thinker.cu) ---- */
#define ORC_MAX_FEATURES 32
typedef struct orc_evaluator orc_evaluator;
/* features[n] square masks; values = the tables of all features in order
 * (3^popcount(mask) doubles each, as in the reference's value file) and
 * the offset.  Returns NULL on bad arguments or allocation failure. */
orc_evaluator* orc_eval_create(const uint64_t* features, int n, const double* values,
                               double offset);
void orc_eval_free(orc_evaluator* ev);
/* Evaluator::eval (eval.cu:129-141): me = side to move. */
float orc_eval(const orc_evaluator* ev, uint64_t me, uint64_t op);
/* think_kernel's search of one position to `depth` plies (>= 4): returns
 * the value; *best = the root's best move (64 = pass); *steps = the
 * reference's loop-step count; *nodes = root, children, pass frames and
 * leaves. */
int orc_think(const orc_evaluator* ev, uint64_t p, uint64_t o, int depth, int* best,
              uint64_t* steps, uint64_t* nodes);
int orc_think_batch(const orc_evaluator* ev, const uint64_t* p, const uint64_t* o, int n,
                    int depth, int threads, int8_t* score, int8_t* best, uint64_t* steps,
                    uint64_t* nodes);

#ifdef __cplusplus
}
#endif
#endif
