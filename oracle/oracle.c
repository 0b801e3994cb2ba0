/*
 * CPU oracle for the batched exact endgame solver -- TEST INFRASTRUCTURE.
 * See oracle.h for who may use it.  Every function cites the reference
 * behaviour it restates (paths are within the reference project).
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static int popc(uint64_t x) { return __builtin_popcountll(x); }
static int ctz(uint64_t x) { return x ? __builtin_ctzll(x) : 64; }
static int clz(uint64_t x) { return x ? __builtin_clzll(x) : 64; }

/* ------------------------------------------------------------------ */
/* Ray tables: for every square and each of the 8 compass directions, the
 * squares strictly beyond it in that direction (built by walking the grid,
 * so they do not depend on any shift-mask constant). */
static const int DR[8] = {0, 0, 1, -1, 1, 1, -1, -1};
static const int DC[8] = {1, -1, 0, 0, 1, -1, 1, -1};
static uint64_t g_ray[64][8];
static pthread_once_t g_once = PTHREAD_ONCE_INIT;

static void init_tables(void) {
  for (int sq = 0; sq < 64; ++sq) {
    for (int d = 0; d < 8; ++d) {
      uint64_t m = 0;
      int r = sq / 8 + DR[d], c = sq % 8 + DC[d];
      while (r >= 0 && r < 8 && c >= 0 && c < 8) {
        m |= 1ULL << (r * 8 + c);
        r += DR[d];
        c += DC[d];
      }
      g_ray[sq][d] = m;
    }
  }
}
static void ensure_tables(void) { pthread_once(&g_once, init_tables); }

/* Flipped discs for a move at `sq` (board.cu:28-54 semantics: the discs of
 * `o` bracketed between sq and a disc of `p` on each of the 8 rays).
 * Rays going to higher bit numbers meet their nearest square at the lowest
 * bit, rays going to lower bit numbers at the highest bit. */
uint64_t orc_flip(uint64_t p, uint64_t o, int sq) {
  ensure_tables();
  uint64_t flipped = 0;
  for (int d = 0; d < 8; ++d) {
    const uint64_t ray = g_ray[sq][d];
    const uint64_t stop = ray & ~o; /* first non-opponent square ends the run */
    if (!stop) continue;
    const int up = (DR[d] * 8 + DC[d]) > 0;
    const uint64_t near = up ? (stop & (0 - stop)) : (1ULL << (63 - clz(stop)));
    if (!(near & p)) continue;
    flipped |= up ? (ray & (near - 1)) : (ray & ~((near << 1) - 1));
  }
  return flipped;
}

/* Independent 8-direction walk, used only to cross-check orc_flip. */
uint64_t orc_flip_naive(uint64_t p, uint64_t o, int sq) {
  uint64_t flipped = 0;
  for (int d = 0; d < 8; ++d) {
    uint64_t run = 0;
    int r = sq / 8 + DR[d], c = sq % 8 + DC[d];
    while (r >= 0 && r < 8 && c >= 0 && c < 8) {
      const uint64_t b = 1ULL << (r * 8 + c);
      if (o & b) {
        run |= b;
      } else {
        if (p & b) flipped |= run;
        break;
      }
      r += DR[d];
      c += DC[d];
    }
  }
  return flipped;
}

/* Legal-move mask (board.cu:56-78 semantics): empty squares from which some
 * ray crosses one or more opponent discs and ends on a player disc.
 * Restated as plain shift propagation per direction. */
uint64_t orc_mobility(uint64_t p, uint64_t o) {
  const uint64_t notA = 0xfefefefefefefefeULL; /* excludes column A */
  const uint64_t notH = 0x7f7f7f7f7f7f7f7fULL; /* excludes column H */
  const uint64_t empty = ~(p | o);
  uint64_t moves = 0;
  /* shift amount, and the mask applied after shifting left / right */
  const int sh[4] = {1, 8, 7, 9};
  const uint64_t ml[4] = {notA, ~0ULL, notH, notA};
  const uint64_t mr[4] = {notH, ~0ULL, notA, notH};
  for (int d = 0; d < 4; ++d) {
    uint64_t t = o & ((p << sh[d]) & ml[d]);
    for (int k = 0; k < 5; ++k) t |= o & ((t << sh[d]) & ml[d]);
    moves |= (t << sh[d]) & ml[d];
    t = o & ((p >> sh[d]) & mr[d]);
    for (int k = 0; k < 5; ++k) t |= o & ((t >> sh[d]) & mr[d]);
    moves |= (t >> sh[d]) & mr[d];
  }
  return moves & empty;
}

uint64_t orc_mobility_naive(uint64_t p, uint64_t o) {
  uint64_t moves = 0, empty = ~(p | o);
  for (int sq = 0; sq < 64; ++sq)
    if (((empty >> sq) & 1) && orc_flip_naive(p, o, sq)) moves |= 1ULL << sq;
  return moves;
}

/* Disc difference at game end with the empties awarded to the winner
 * (board.cuh:7-18). */
int orc_final_score(uint64_t p, uint64_t o) {
  const int pc = popc(p), oc = popc(o);
  if (pc == oc) return 0;
  if (pc > oc) return 64 - 2 * oc;
  return 2 * pc - 64;
}

/* ------------------------------------------------------------------ */
/* base81 codec.  Char i covers squares 4i..4i+3; square j of the group adds
 * w_j for the player and 2*w_j for the opponent, w = {1,3,9,32}, plus 33
 * (test.cpp:7-19; to_board.cpp:15-39 is its inverse). */
void orc_encode(uint64_t p, uint64_t o, char out[17]) {
  static const int w[4] = {1, 3, 9, 32};
  for (int i = 0; i < 16; ++i) {
    int v = 33;
    for (int j = 0; j < 4; ++j) {
      const int sq = 4 * i + j;
      if ((p >> sq) & 1) v += w[j];
      if ((o >> sq) & 1) v += 2 * w[j];
    }
    out[i] = (char)v;
  }
  out[16] = '\0';
}

int orc_decode(const char* s, uint64_t* p, uint64_t* o) {
  uint64_t pp = 0, oo = 0;
  for (int i = 0; i < 16; ++i) {
    const int v = (int)(unsigned char)s[i] - 33;
    if (v < 0 || v > 90) return -1;
    const int hi = v >> 5, lo = v & 31;
    if (hi > 2 || lo > 26) return -1;
    const int digit[4] = {lo % 3, (lo / 3) % 3, lo / 9, hi};
    for (int j = 0; j < 4; ++j) {
      const uint64_t b = 1ULL << (4 * i + j);
      if (digit[j] == 1) pp |= b;
      if (digit[j] == 2) oo |= b;
    }
  }
  *p = pp;
  *o = oo;
  return 0;
}

/* ------------------------------------------------------------------ */
/* Position generator.
 *   state: xoshiro256** seeded with four successive splitmix64 outputs
 *          starting from x0 = (seed << 32) + index;
 *   uniform(k) = high 64 bits of next() * k;
 *   if min != max: empties E = min + uniform(max - min + 1), drawn first;
 *   play from the standard start (black to move, black d5/e4, white d4/e5):
 *     - when exactly E squares are empty, emit (side to move, other side);
 *     - else if the side to move has k legal moves, play the uniform(k)-th
 *       set bit of the move mask counting from bit 0;
 *     - else if only the other side can move, pass;
 *     - else (game over before E) restart from the start position,
 *       continuing the same PRNG stream. */
static uint64_t splitmix64(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
typedef struct { uint64_t s[4]; } xoshiro;
static uint64_t xo_next(xoshiro* r) {
  uint64_t* s = r->s;
  const uint64_t result = rotl(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl(s[3], 45);
  return result;
}
static uint64_t xo_uniform(xoshiro* r, uint64_t k) {
  return (uint64_t)(((unsigned __int128)xo_next(r) * k) >> 64);
}

void orc_generate(uint64_t seed, uint64_t first_index, int n, int min_empties,
                  int max_empties, uint64_t* out_p, uint64_t* out_o) {
  const uint64_t black0 = 0x0000000810000000ULL, white0 = 0x0000001008000000ULL;
  for (int i = 0; i < n; ++i) {
    uint64_t x = (seed << 32) + first_index + (uint64_t)i;
    xoshiro r;
    for (int k = 0; k < 4; ++k) r.s[k] = splitmix64(&x);
    int target = min_empties;
    if (max_empties > min_empties)
      target = min_empties + (int)xo_uniform(&r, (uint64_t)(max_empties - min_empties + 1));
    uint64_t p = black0, o = white0;
    for (;;) {
      if (64 - popc(p | o) == target) break;
      uint64_t moves = orc_mobility(p, o);
      if (!moves) {
        if (orc_mobility(o, p)) {
          uint64_t t = p;
          p = o;
          o = t;
        } else {
          p = black0;
          o = white0;
        }
        continue;
      }
      uint64_t j = xo_uniform(&r, (uint64_t)popc(moves));
      while (j--) moves &= moves - 1;
      const int sq = ctz(moves);
      const uint64_t f = orc_flip(p, o, sq);
      const uint64_t np = o ^ f, no = p ^ f ^ (1ULL << sq);
      p = np;
      o = no;
    }
    out_p[i] = p;
    out_o[i] = o;
  }
}

/* ------------------------------------------------------------------ */
/* Reference-order search.  Mirrors the reference's state machine
 * (solver.cu:162-283) node for node so that both its score and its loop-step
 * count can be checked against the reference:
 *   - plies 0 .. depth-10 are "upper" nodes: legal moves in empty-scan order
 *     (corners first, then lowest square; node.cuh:21-28) stably sorted by
 *     the opponent's move count after the move (solver.cu:78-93);
 *   - deeper plies are "lower" nodes that try every empty square in the same
 *     scan order and skip the ones that flip nothing (solver.cu:244-270);
 *   - fail-soft commit: result = max(result, v), alpha = max(alpha, result)
 *     (node.cuh:70-73, solver.cu:146-149), cut when alpha >= beta;
 *   - a side without moves passes in place with the window negated and
 *     swapped; a second pass scores the position (solver.cu:65-73, 214-221,
 *     246-256), and the parent takes +result from a passed child
 *     (solver.cu:57-61, 183, 200).
 * Each function returns the value from the point of view of the side to
 * move when the node was created. */
typedef struct {
  uint64_t steps, nodes;
  int upper_size;
} ref_ctx;

static uint64_t scan_next(uint64_t* unchecked) {
  const uint64_t corner = 0x8100000000000081ULL;
  const uint64_t c = *unchecked & corner;
  const uint64_t bit = c ? (c & (0 - c)) : (*unchecked & (0 - *unchecked));
  *unchecked ^= bit;
  return bit;
}

static int ref_lower(ref_ctx* cx, uint64_t p, uint64_t o, int alpha, int beta) {
  cx->nodes++;
  int passed = 0;
  for (;;) {
    int result = -32767, found = 0;
    uint64_t unchecked = ~(p | o);
    while (unchecked) {
      if (alpha >= beta) {
        cx->steps++;
        return passed ? -result : result;
      }
      cx->steps++;
      const uint64_t bit = scan_next(&unchecked);
      const uint64_t f = orc_flip(p, o, ctz(bit));
      if (f) {
        found = 1;
        const int v = -ref_lower(cx, o ^ f, p ^ f ^ bit, -beta, -alpha);
        if (v > result) result = v;
        if (result > alpha) alpha = result;
      }
    }
    if (found) {
      cx->steps++;
      return passed ? -result : result;
    }
    cx->steps++;
    if (passed) {
      result = orc_final_score(p, o);
      return -result;
    }
    cx->nodes++; /* the pass frame */
    passed = 1;
    const uint64_t t = p;
    p = o;
    o = t;
    const int a = alpha;
    alpha = -beta;
    beta = -a;
  }
}

typedef struct {
  int n;
  uint8_t sq[46];
} move_list;

static void upper_moves(uint64_t p, uint64_t o, move_list* ml) {
  int8_t key[46];
  uint64_t unchecked = ~(p | o);
  ml->n = 0;
  while (unchecked) {
    const uint64_t bit = scan_next(&unchecked);
    const int sq = ctz(bit);
    const uint64_t f = orc_flip(p, o, sq);
    if (f) {
      key[ml->n] = (int8_t)popc(orc_mobility(o ^ f, p ^ f ^ bit));
      ml->sq[ml->n++] = (uint8_t)sq;
    }
  }
  for (int i = 1; i < ml->n; ++i) { /* stable insertion sort by key */
    const int8_t k = key[i];
    const uint8_t s = ml->sq[i];
    int j = i - 1;
    while (j >= 0 && k < key[j]) {
      key[j + 1] = key[j];
      ml->sq[j + 1] = ml->sq[j];
      --j;
    }
    key[j + 1] = k;
    ml->sq[j + 1] = s;
  }
}

static int ref_upper(ref_ctx* cx, uint64_t p, uint64_t o, int alpha, int beta, int ply) {
  cx->nodes++;
  move_list ml;
  int passed = 0;
  upper_moves(p, o, &ml);
  if (ml.n == 0) {
    cx->steps++; /* pass_upper */
    cx->nodes++;
    passed = 1;
    const uint64_t t = p;
    p = o;
    o = t;
    const int a = alpha;
    alpha = -beta;
    beta = -a;
    upper_moves(p, o, &ml);
    if (ml.n == 0) {
      cx->steps++;
      return -orc_final_score(p, o);
    }
  }
  int result = -64;
  for (int i = 0; i < ml.n; ++i) {
    if (alpha >= beta) break;
    cx->steps++;
    const uint64_t bit = 1ULL << ml.sq[i];
    const uint64_t f = orc_flip(p, o, ml.sq[i]);
    int v;
    if (ply + 1 < cx->upper_size)
      v = -ref_upper(cx, o ^ f, p ^ f ^ bit, -beta, -alpha, ply + 1);
    else
      v = -ref_lower(cx, o ^ f, p ^ f ^ bit, -beta, -alpha);
    if (v > result) result = v;
    if (result > alpha) alpha = result;
  }
  cx->steps++;
  return passed ? -result : result;
}

int orc_solve_ref(uint64_t p, uint64_t o, int depth, uint64_t* steps, uint64_t* nodes) {
  ensure_tables();
  ref_ctx cx = {0, 0, depth - 9};
  const int v = ref_upper(&cx, p, o, -64, 64, 0);
  if (steps) *steps = cx.steps;
  if (nodes) *nodes = cx.nodes;
  return v;
}

/* ------------------------------------------------------------------ */
/* Independent fast solver: fail-soft alpha-beta over the legal-move mask,
 * fastest-first ordering (fewest opponent replies, corners preferred) at 6+
 * empties, corners-then-lowest below.  Shares only orc_flip/orc_mobility. */
static int fast_search(uint64_t p, uint64_t o, int alpha, int beta, uint64_t* nodes, int* best) {
  (*nodes)++;
  uint64_t moves = orc_mobility(p, o);
  if (!moves) {
    if (!orc_mobility(o, p)) {
      if (best) *best = 65;
      return orc_final_score(p, o);
    }
    if (best) *best = 64;
    return -fast_search(o, p, -beta, -alpha, nodes, NULL);
  }
  const int empties = 64 - popc(p | o);
  uint8_t sq[32];
  int key[32], n = 0;
  while (moves) {
    const uint64_t bit = moves & (0 - moves);
    moves ^= bit;
    const int s = ctz(bit);
    int k = 0;
    if (empties >= 6) {
      const uint64_t f = orc_flip(p, o, s);
      k = popc(orc_mobility(o ^ f, p ^ f ^ bit)) * 16;
      if (bit & 0x8100000000000081ULL) k -= 8;
    } else {
      k = (bit & 0x8100000000000081ULL) ? 0 : 1;
    }
    int j = n++;
    while (j > 0 && key[j - 1] > k) {
      key[j] = key[j - 1];
      sq[j] = sq[j - 1];
      --j;
    }
    key[j] = k;
    sq[j] = (uint8_t)s;
  }
  int bestv = -65, bestm = sq[0];
  for (int i = 0; i < n; ++i) {
    const uint64_t bit = 1ULL << sq[i];
    const uint64_t f = orc_flip(p, o, sq[i]);
    const int a = alpha > bestv ? alpha : bestv;
    const int v = -fast_search(o ^ f, p ^ f ^ bit, -beta, -a, nodes, NULL);
    if (v > bestv) {
      bestv = v;
      bestm = sq[i];
      if (v >= beta) break;
    }
  }
  if (best) *best = bestm;
  return bestv;
}

int orc_solve_fast(uint64_t p, uint64_t o, uint64_t* nodes, int* best) {
  ensure_tables();
  uint64_t cnt = 0;
  int b = 65;
  const int v = fast_search(p, o, -64, 64, &cnt, &b);
  if (nodes) *nodes = cnt;
  if (best) *best = b;
  return v;
}

/* ------------------------------------------------------------------ */
typedef struct {
  const uint64_t *p, *o;
  int n, depth, mode;
  int8_t* score;
  uint64_t *steps, *nodes;
  int8_t* best;
  int next;
} batch_job;

static void* batch_worker(void* arg) {
  batch_job* job = (batch_job*)arg;
  for (;;) {
    const int i = __atomic_fetch_add(&job->next, 1, __ATOMIC_RELAXED);
    if (i >= job->n) break;
    uint64_t st = 0, nd = 0;
    int v, b = 65;
    if (job->mode == 0)
      v = orc_solve_ref(job->p[i], job->o[i], job->depth, &st, &nd);
    else
      v = orc_solve_fast(job->p[i], job->o[i], &nd, &b);
    job->score[i] = (int8_t)v;
    if (job->steps) job->steps[i] = st;
    if (job->nodes) job->nodes[i] = nd;
    if (job->best) job->best[i] = (int8_t)b;
  }
  return NULL;
}

int orc_num_cores(void) {
  long c = sysconf(_SC_NPROCESSORS_ONLN);
  return c > 0 ? (int)c : 1;
}

int orc_solve_batch(const uint64_t* p, const uint64_t* o, int n, int depth, int mode,
                    int threads, int8_t* score, uint64_t* steps, uint64_t* nodes, int8_t* best) {
  ensure_tables();
  if (threads <= 0) threads = orc_num_cores();
  if (threads > 256) threads = 256;
  batch_job job = {p, o, n, depth, mode, score, steps, nodes, best, 0};
  pthread_t tid[256];
  for (int t = 1; t < threads; ++t) pthread_create(&tid[t], NULL, batch_worker, &job);
  batch_worker(&job);
  for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Pattern evaluator (eval.cu:12-141).  A feature is a square mask; its
 * table has 3^k entries for k = popcount(mask), indexed by the base-3
 * number whose digit j is 0 (empty), 1 (`me`) or 2 (`op`) on the mask's
 * j-th lowest square (eval.cu:81-89, 107-113: base3[pext(me)] +
 * 2 base3[pext(op)]).  The board is scored in all 8 symmetries: 4 rotations
 * (rot90 = vertical flip after the A1-H8 transpose, eval.cu:102-104), each
 * as is and transposed, features in file order, summed in float in exactly
 * that order, plus the offset, clamped to [-64, 64] (eval.cu:129-141).
 * Table values are read as doubles and stored as float (eval.cu:44-46). */
struct orc_evaluator {
  int n;
  uint64_t feature[ORC_MAX_FEATURES];
  float* value[ORC_MAX_FEATURES];
  float offset;
};

static int pow3i(int k) {
  int r = 1;
  while (k-- > 0) r *= 3;
  return r;
}

orc_evaluator* orc_eval_create(const uint64_t* features, int n, const double* values,
                               double offset) {
  if (n < 0 || n > ORC_MAX_FEATURES) return NULL;
  orc_evaluator* ev = (orc_evaluator*)calloc(1, sizeof(orc_evaluator));
  if (!ev) return NULL;
  ev->n = n;
  size_t off = 0;
  for (int j = 0; j < n; ++j) {
    ev->feature[j] = features[j];
    const int len = pow3i(popc(features[j]));
    ev->value[j] = (float*)malloc(sizeof(float) * (size_t)len);
    for (int i = 0; i < len; ++i) ev->value[j][i] = (float)values[off + (size_t)i];
    off += (size_t)len;
  }
  ev->offset = (float)offset;
  return ev;
}

void orc_eval_free(orc_evaluator* ev) {
  if (!ev) return;
  for (int j = 0; j < ev->n; ++j) free(ev->value[j]);
  free(ev);
}

/* base-3 index of the mask's squares: digit 1 for `me`, 2 for `op` */
static int feature_index(uint64_t me, uint64_t op, uint64_t mask) {
  int idx = 0, w = 1;
  while (mask) {
    const uint64_t b = mask & (0 - mask);
    mask ^= b;
    if (me & b) idx += w;
    if (op & b) idx += 2 * w;
    w *= 3;
  }
  return idx;
}

/* transpose about the A1-H8 diagonal: square (r, c) -> (c, r) */
static uint64_t transpose(uint64_t x) {
  uint64_t y = 0;
  for (int sq = 0; sq < 64; ++sq)
    if ((x >> sq) & 1) y |= 1ULL << ((sq % 8) * 8 + sq / 8);
  return y;
}

/* vertical flip: row r -> row 7 - r */
static uint64_t flip_rows(uint64_t x) {
  uint64_t y = 0;
  for (int r = 0; r < 8; ++r) y |= ((x >> (8 * r)) & 0xFF) << (8 * (7 - r));
  return y;
}

float orc_eval(const orc_evaluator* ev, uint64_t me, uint64_t op) {
  float score = 0.0f;
  for (int i = 0; i < 4; ++i) {
    const uint64_t tme = transpose(me), top = transpose(op);
    for (int j = 0; j < ev->n; ++j) {
      score += ev->value[j][feature_index(me, op, ev->feature[j])];
      score += ev->value[j][feature_index(tme, top, ev->feature[j])];
    }
    me = flip_rows(tme);
    op = flip_rows(top);
  }
  const float s = score + ev->offset;
  return s > 64.0f ? 64.0f : (s < -64.0f ? -64.0f : s);
}

/* ------------------------------------------------------------------ */
/* Think mode (thinker.cu:12-376): depth-limited fail-soft negamax.  The
 * first depth-3 plies are "upper" nodes (thinker.cu:14-107): legal moves
 * ordered by the opponent's move count after the move, stably, from the
 * corners-first scan; result starts at -65 and a commit that raises it
 * records the move (thinker.cu:97-103).  The last 3 plies are the
 * reference's lower nodes (node.cuh:56-74, thinker.cu:226-262), as in the
 * solve path.  A move at the last lower ply reaches a leaf scored
 * round(eval(leaf)) (thinker.cu:324-326, 200-204); a game that ends before
 * that depth is scored exactly.  Passes take no ply.  The root's best move
 * is 64 (pass) when the root passed (thinker.cu:167-170).  Steps count the
 * reference's loop iterations (thinker.cu:321-335); nodes count the root,
 * every pushed child, pass frame and leaf. */
typedef struct {
  const orc_evaluator* ev;
  int upper_size, depth;
  uint64_t steps, nodes;
} think_ctx;

static int think_lower(think_ctx* cx, uint64_t p, uint64_t o, int alpha, int beta, int level) {
  cx->nodes++;
  int passed = 0;
  for (;;) {
    int result = -32767, found = 0;
    uint64_t unchecked = ~(p | o);
    while (unchecked) {
      if (alpha >= beta) {
        cx->steps++;
        return passed ? -result : result;
      }
      cx->steps++;
      const uint64_t bit = scan_next(&unchecked);
      const uint64_t f = orc_flip(p, o, ctz(bit));
      if (f) {
        found = 1;
        int v;
        if (level == cx->depth - 1) {
          cx->steps++; /* the leaf's own step */
          cx->nodes++;
          v = -(int)roundf(orc_eval(cx->ev, o ^ f, p ^ f ^ bit));
        } else {
          v = -think_lower(cx, o ^ f, p ^ f ^ bit, -beta, -alpha, level + 1);
        }
        if (v > result) result = v;
        if (result > alpha) alpha = result;
      }
    }
    if (found) {
      cx->steps++;
      return passed ? -result : result;
    }
    cx->steps++;
    if (passed) return -orc_final_score(p, o);
    cx->nodes++; /* the pass frame */
    passed = 1;
    const uint64_t t = p;
    p = o;
    o = t;
    const int a = alpha;
    alpha = -beta;
    beta = -a;
  }
}

static int think_upper(think_ctx* cx, uint64_t p, uint64_t o, int alpha, int beta, int ply,
                       int* best) {
  cx->nodes++;
  move_list ml;
  int passed = 0;
  upper_moves(p, o, &ml);
  if (ml.n == 0) {
    cx->steps++; /* pass_upper */
    cx->nodes++;
    passed = 1;
    const uint64_t t = p;
    p = o;
    o = t;
    const int a = alpha;
    alpha = -beta;
    beta = -a;
    upper_moves(p, o, &ml);
    if (ml.n == 0) {
      cx->steps++;
      *best = 64;
      return -orc_final_score(p, o);
    }
  }
  int result = -65, bm = 65, child_best = 65;
  for (int i = 0; i < ml.n; ++i) {
    if (alpha >= beta) break;
    cx->steps++;
    const uint64_t bit = 1ULL << ml.sq[i];
    const uint64_t f = orc_flip(p, o, ml.sq[i]);
    int v;
    if (ply + 1 < cx->upper_size)
      v = -think_upper(cx, o ^ f, p ^ f ^ bit, -beta, -alpha, ply + 1, &child_best);
    else
      v = -think_lower(cx, o ^ f, p ^ f ^ bit, -beta, -alpha, ply + 1);
    if (v > result) {
      result = v;
      bm = ml.sq[i];
      if (result > alpha) alpha = result;
    }
  }
  cx->steps++;
  *best = passed ? 64 : bm;
  return passed ? -result : result;
}

int orc_think(const orc_evaluator* ev, uint64_t p, uint64_t o, int depth, int* best,
              uint64_t* steps, uint64_t* nodes) {
  ensure_tables();
  think_ctx cx = {ev, depth - 3, depth, 0, 0};
  int b = 65;
  const int v = think_upper(&cx, p, o, -64, 64, 0, &b);
  if (best) *best = b;
  if (steps) *steps = cx.steps;
  if (nodes) *nodes = cx.nodes;
  return v;
}

typedef struct {
  const orc_evaluator* ev;
  const uint64_t *p, *o;
  int n, depth;
  int8_t *score, *best;
  uint64_t *steps, *nodes;
  int next;
} think_job;

static void* think_worker(void* arg) {
  think_job* job = (think_job*)arg;
  for (;;) {
    const int i = __atomic_fetch_add(&job->next, 1, __ATOMIC_RELAXED);
    if (i >= job->n) break;
    uint64_t st = 0, nd = 0;
    int b = 65;
    const int v = orc_think(job->ev, job->p[i], job->o[i], job->depth, &b, &st, &nd);
    job->score[i] = (int8_t)v;
    if (job->best) job->best[i] = (int8_t)b;
    if (job->steps) job->steps[i] = st;
    if (job->nodes) job->nodes[i] = nd;
  }
  return NULL;
}

int orc_think_batch(const orc_evaluator* ev, const uint64_t* p, const uint64_t* o, int n,
                    int depth, int threads, int8_t* score, int8_t* best, uint64_t* steps,
                    uint64_t* nodes) {
  ensure_tables();
  if (depth < 4) return -1;
  if (threads <= 0) threads = orc_num_cores();
  if (threads > 256) threads = 256;
  think_job job = {ev, p, o, n, depth, score, best, steps, nodes, 0};
  pthread_t tid[256];
  for (int t = 1; t < threads; ++t) pthread_create(&tid[t], NULL, think_worker, &job);
  think_worker(&job);
  for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
  return 0;
}
