// Batched solver: one persistent launch over a device work queue of
// positions ordered by empty count (most empties first).  A lane searches
// one position at a time and refills itself from the queue; when the queue
// is empty (or the warp already holds its quota of positions) idle lanes
// help the busy lanes of their own warp with their positions.
//
// Search (values identical to the reference's negamax, solver.cu:15-283;
// the tree differs):
//   - fail-soft principal-variation search: the first move of a node gets
//     the node's window, later moves a null window just above the best value
//     so far, and a move that beats it is searched again with the window
//     above it;
//   - move order: nodes with >= ff empties play their moves by fewest
//     opponent replies (corners first on ties) from a packed five-entry list
//     (the role of the reference's sorted UpperNode list, solver.cu:78-93);
//     below ff, corners, then squares of odd-parity quadrants, avoiding
//     X-squares;
//   - transposition table (table.cuh) at nodes with >= tt_min empties: a
//     probe when the node is created (a bound outside the window closes it,
//     one inside narrows the window) and a bound stored when it closes;
//   - stability cutoff at nodes with >= stab_min empties and alpha >=
//     stab_gate + 3 * empties: discs of the opponent that can never flip cap
//     the side to move's score at 64 - 2 * stable, which closes a node whose
//     alpha is at or above it (lopsided positions, the slowest to solve,
//     gain most);
//   - a move at a node with two empties scores its child (one empty) in the
//     same step: the child's last move needs only a flip count;
//   - passes happen in place with the window negated and swapped
//     (solver.cu:57-73, 214-221, 246-256 semantics); the position after
//     the pass is a node of its own for the table and the stability cutoff
//     (in a lopsided game one side passes again and again).
//
// Uniform step.  Every loop iteration every lane does at most one move flip
// plus one mobility (or, at nodes with two empties, the child's last-square
// flip counts from two small table lookups per line):
// a move (the child is pushed), a fastest-first ordering probe, a root init,
// a pass, a re-mask, or a handed-out move.  Only the bookkeeping around it
// diverges.  The loop keeps one copy of the flip and of the mobility code,
// and the rare paths (table, stability, split-node search) out of line: the
// hot loop's instruction footprint decides how often warps wait for
// instruction fetch.
//
// Frames: a node with E empties saves {move word, flips of the move being
// searched, packed alpha/beta/best/square/flags} in slot E when it pushes a
// child; a node with two empties never pushes, so slots run 3..depth.  All
// slots live in shared memory, interleaved by thread ([slot][thread]), when
// they fit, else in a per-lane global array.  Bit 0 of the flips word (A1,
// a corner, which is never flipped) records that the child is being
// searched again after beating a null window.
//
// Helping (young brothers wait, inside one warp).  A lane may offer one of
// its nodes as a split node: >= help_min empties, not passed, first move
// searched (that is the "young brothers wait" condition), window still open,
// moves left in its frame.  While the owner is below that node, idle lanes
// of the warp receive its untried moves, one per idle lane and iteration;
// the owner lane itself takes each move from its own frame, so the frame has
// one writer.  A helper searches the child with a null window above the
// node's best value, searches it again with the window above its result when
// it beats that bound, and reports the value with atomicMax into the owner's
// result word (value, exactness, move) and a count of outstanding moves.  An
// owner closes its split node only after every handed-out move has reported;
// a cutoff (or an abort) at the node raises a flag that makes its helpers
// abandon their subtrees.  Helpers may split their own nodes in turn.  All
// waiting is between lanes of one warp inside one loop, so it always ends;
// a launch deadline still bounds everything.
//
// Tail handoff.  Once the queue is used up and at most tail_count positions
// are unfinished, every warp stops its searches the way the deadline does
// (without the error): each stopped position gets the score kUnsolvedDev and
// its root's lower bound (the best value of its completed moves), and the
// host finishes them with a root split over the whole GPU.  Roots may carry
// windows (root_window): the root split searches its frontier with windows
// derived from those bounds.
#include "common.cuh"
#include "kernels.h"
#include "search.cuh"
#include "table.cuh"

namespace gpo {

namespace {

enum : int { OP_NONE = 0, OP_INIT, OP_MOVE, OP_PASS, OP_KEY, OP_REMASK, OP_HAND };
enum : int { PH_INIT = 0, PH_MASK, PH_KEY, PH_LIST };

// shared tables: 64 x 4 up-rays (flip), 64 x 2 diagonal masks and the
// 8 x 256 last-square flip counts (bitboard.cuh)
constexpr int kTableBytes = (256 + 128) * 8 + 8 * 256;
constexpr unsigned kFull = 0xffffffffu;
constexpr u64 kResearch = 1ULL;  // flips-word flag: the child is a re-search
// Levels a lane may return through per iteration.  A lane finishing a deep
// subtree can return through several levels at once; every extra level is
// another pass of the warp through the return code, so a lane with more to
// return continues in the next iteration instead.
constexpr int kMaxPops = 2;

__device__ __forceinline__ unsigned pack_meta(int sq, int alpha, int beta, int best, int passed,
                                              int list) {
  return static_cast<unsigned>(sq) | (static_cast<unsigned>(alpha & 0xff) << 6) |
         (static_cast<unsigned>(beta & 0xff) << 14) | (static_cast<unsigned>(best & 0xff) << 22) |
         (static_cast<unsigned>(passed) << 30) | (static_cast<unsigned>(list) << 31);
}
__device__ __forceinline__ int meta_sq(unsigned x) { return static_cast<int>(x & 63u); }
__device__ __forceinline__ int meta_alpha(unsigned x) {
  return static_cast<signed char>((x >> 6) & 0xff);
}
__device__ __forceinline__ int meta_beta(unsigned x) {
  return static_cast<signed char>((x >> 14) & 0xff);
}
__device__ __forceinline__ int meta_best(unsigned x) {
  return static_cast<signed char>((x >> 22) & 0xff);
}
__device__ __forceinline__ int meta_passed(unsigned x) { return static_cast<int>((x >> 30) & 1u); }
__device__ __forceinline__ int meta_list(unsigned x) { return static_cast<int>(x >> 31); }

// Helper results: (value + 128) << 9 | exact << 8 | move; 0 = none.  The
// max prefers the higher value, then an exact value over a bound.
__device__ __forceinline__ unsigned pack_acc(int v, int exact, int move) {
  return (static_cast<unsigned>(v + 128) << 9) | (static_cast<unsigned>(exact) << 8) |
         static_cast<unsigned>(move & 255);
}
__device__ __forceinline__ int acc_value(unsigned a) { return static_cast<int>(a >> 9) - 128; }

// Frame slots 3..depth of one lane: all in shared memory ([slot][thread])
// when they fit beside the launch's occupancy, else all in the global frame
// array ([slot][grid thread], L1-cached).  One address formula for both,
// used through generic loads and stores.
struct Frames {
  u64* m;            // M word of slot E: m[E * stride + off]
  u64* f;            // F words, same indexing
  unsigned* x;       // X words, same indexing
  long long stride;  // threads the slots are interleaved over
  long long off;     // this thread's index minus 3 * stride

  __device__ __forceinline__ long long idx(int E) const { return E * stride + off; }
  __device__ __forceinline__ u64* m_ptr(int E) const { return m + idx(E); }
  __device__ __forceinline__ u64* f_ptr(int E) const { return f + idx(E); }
  __device__ __forceinline__ void store(int E, u64 mv, u64 fv, unsigned xv) const {
    const long long i = idx(E);
    m[i] = mv;
    f[i] = fv;
    x[i] = xv;
  }
  __device__ __forceinline__ void load(int E, u64& mv, u64& fv, unsigned& xv) const {
    const long long i = idx(E);
    mv = m[i];
    fv = f[i];
    xv = x[i];
  }
};

// Per-lane split-node state in shared memory, read by the lanes that help.
struct SplitState {
  u64* P;            // position of the split node
  u64* O;
  unsigned* pend;    // handed-out moves not yet reported
  unsigned* acc;     // best helper result (pack_acc), 0 = none
  unsigned* cut;     // 1 = the node was cut off or abandoned: helpers stop
  int* lo;           // owner's best lower bound at the node (max(alpha, best))
  int* beta;
};

__device__ __forceinline__ unsigned ld_shared_volatile(const unsigned* p) {
  return *reinterpret_cast<const volatile unsigned*>(p);
}
__device__ __forceinline__ int ld_shared_volatile(const int* p) {
  return *reinterpret_cast<const volatile int*>(p);
}
__device__ __forceinline__ unsigned ld_global_volatile(const unsigned* p) {
  return *reinterpret_cast<const volatile unsigned*>(p);
}

// k-th (0-based) set bit of m, m having more than k bits set.
__device__ __forceinline__ int nth_bit(unsigned m, int k) {
  for (int i = 0; i < k; ++i) m &= m - 1u;
  return __ffs(static_cast<int>(m)) - 1;
}

// ---- table access, and the rare paths kept out of line so that the hot
//      loop stays small ----

// Table bounds of (P, O): 0 = not found, else 1 << 16 | (lower + 64) << 8 |
// (upper + 64).
__device__ __forceinline__ unsigned tt_lookup(unsigned long long* tt, int bits, u64 P, u64 O) {
  int lb, ub;
  if (!tt_probe(tt, bits, tt_key(P, O), lb, ub)) return 0u;
  return (1u << 16) | (static_cast<unsigned>(lb + 64) << 8) | static_cast<unsigned>(ub + 64);
}

// Stores the bound a closed node proves: best >= beta proves value >= best,
// anything lower proves value <= best (an exact value is also an upper
// bound).  Returns 1 if stored.
__device__ __forceinline__ int tt_record(unsigned long long* tt, int bits, u64 P, u64 O, int best,
                                      int beta) {
  const TTKey k = tt_key(P, O);
  return best >= beta ? tt_store(tt, bits, k, best, 64) : tt_store(tt, bits, k, -64, best);
}

__device__ __noinline__ int stable_count(u64 O, u64 occ) { return popc(gpo_stable(O, occ)); }

// The learned move list of (P, O) from the order table, or 0 (mlp.cu fills
// the table with linear probing from the key's bucket, at most 16 slots).
__device__ __noinline__ u64 order_lookup(const u64* table, int bits, u64 P, u64 O) {
  const TTKey k = tt_key(P, O);
  const size_t mask = (static_cast<size_t>(1) << bits) - 1;
  size_t h = static_cast<size_t>(k.y >> (64 - bits));
  for (int probe = 0; probe < 16; ++probe, h = (h + 1) & mask) {
    const u64* e = table + 4 * h;
    const u64 x = e[0], y = e[1];
    if (x == k.x && y == k.y) return e[2];
    if ((x | y) == 0) return 0;
  }
  return 0;
}

// A lane's split node: the shallowest of its open nodes (slots root_e down
// to E + 1) with >= help_min empties that is not passed, has searched its
// first move, has an open window and has a move left in its frame.  The
// nodes' positions come from replaying the path from the root with the
// stored flips.  Publishes the node in the split-node state and returns its
// slot, or 0.
__device__ __noinline__ int find_split_node(Frames fr, SplitState sp, int t, u64 X, u64 Y,
                                            int root_e, int E, int help_min) {
  for (int e = root_e; e > E; --e) {
    u64 m, f;
    unsigned meta;
    fr.load(e, m, f, meta);
    const int pas = meta_passed(meta);
    if (pas) {
      const u64 tmp = X;
      X = Y;
      Y = tmp;
    }
    const int b0 = meta_beta(meta), best0 = meta_best(meta), a0 = meta_alpha(meta);
    const int lo0 = a0 > best0 ? a0 : best0;
    const bool has = meta_list(meta) ? list_peek(m) != 0xFFF : m != 0;
    if (e >= help_min && !pas && best0 > -65 && lo0 < b0 && has) {
      sp.P[t] = X;
      sp.O[t] = Y;
      sp.lo[t] = lo0;
      sp.beta[t] = b0;
      sp.acc[t] = 0u;
      sp.cut[t] = 0u;
      sp.pend[t] = 0u;
      return e;
    }
    const u64 ff = f & ~kResearch;
    const u64 cx = Y ^ ff, cy = X ^ ff ^ (1ULL << meta_sq(meta));
    X = cx;
    Y = cy;
  }
  return 0;
}

}  // namespace

__device__ __forceinline__ unsigned long long global_ns() { return gpo_global_ns(); }

// Blocks per SM the register allocation must allow (128-thread blocks).
#ifndef GPO_BATCHED_MIN_BLOCKS
#define GPO_BATCHED_MIN_BLOCKS 1
#endif

__global__ void __launch_bounds__(GPO_BATCHED_MIN_BLOCKS > 1 ? 128 : 256, GPO_BATCHED_MIN_BLOCKS)
    batched_kernel(BatchedArgs args) {
  extern __shared__ __align__(16) u64 smem_raw[];
  const int B = blockDim.x;
  const int t = threadIdx.x;
  u64* const rays = smem_raw;         // 64 x 4 up-rays (bitboard.cuh)
  u64* const dmask = smem_raw + 256;  // 64 x 2 diagonal masks
  unsigned char* const lcnt = reinterpret_cast<unsigned char*>(smem_raw + 384);  // 8 x 256 counts
  SplitState sp;
  sp.P = smem_raw + kTableBytes / 8;
  sp.O = sp.P + B;
  sp.pend = reinterpret_cast<unsigned*>(sp.O + B);
  sp.acc = sp.pend + B;
  sp.cut = sp.acc + B;
  sp.lo = reinterpret_cast<int*>(sp.cut + B);
  sp.beta = sp.lo + B;
  u64* const fbase = reinterpret_cast<u64*>(sp.beta + B);  // B is a multiple of 32: aligned
  gpo_build_rays(rays);
  gpo_build_last(lcnt, dmask);
  sp.pend[t] = 0;
  sp.acc[t] = 0;
  sp.cut[t] = 0;
  __syncthreads();

  Frames fr;
  {
    const bool shared = args.depth <= args.smem_top;
    const long long slots = args.depth > 2 ? args.depth - 2 : 0;  // slots 3..depth
    const long long threads = shared ? B : static_cast<long long>(gridDim.x) * B;
    const long long me = shared ? t : static_cast<long long>(blockIdx.x) * B + t;
    fr.m = shared ? fbase : reinterpret_cast<u64*>(args.gframes);
    fr.f = fr.m + slots * threads;
    fr.x = reinterpret_cast<unsigned*>(fr.f + slots * threads);
    fr.stride = threads;
    fr.off = me - 3 * threads;
  }

  const int lane = t & 31;
  const int wbase = t - lane;  // thread index of lane 0 of this warp
  const unsigned lane_lt = (1u << lane) - 1u;
  const unsigned n = static_cast<unsigned>(args.n);
  const int rpw = args.roots_per_warp > 0 ? args.roots_per_warp : 32;
  unsigned long long total_nodes = 0, handouts = 0, stab_cuts = 0;
  unsigned long long tt_probes = 0, tt_hits = 0, tt_updates = 0;

  bool busy = false;    // a search is in progress in this lane
  bool helper = false;  // ... and it is a move handed out by lane `towner`
  bool abort = false;   // close every open node at once, reporting nothing
  bool closed = false;  // the current node was closed when created (table or stability)
  bool qdone = false;   // the input queue is used up (warp-uniform)
  bool late = false;    // the launch deadline has passed, or the tail is handed back (warp-uniform)
  bool handoff = false; // the tail is handed back: open positions end unsolved (warp-uniform)
  unsigned pos = 0;     // input position of the search (the owner's for a helper)
  int towner = 0, tsq = 0, tlo = 0, tbeta = 0;
  bool tres = false;    // a helper's move is being searched again
  int spe = 0;          // slot of this lane's split node, 0 = none
  unsigned chk = 0;
  const unsigned long long deadline = global_ns() + args.wait_limit_ns;
  u64 P = 0, O = 0, moves = 0, lst = 0, P0 = 0, O0 = 0;
  int alpha = 0, beta = 0, best = 0, passed = 0, E = 0, root_e = 0, phase = PH_INIT;
  int rootbest = kMoveNoneDev;
  unsigned long long nodes = 0;

  for (;;) {
    __syncwarp();
    ++chk;
    if ((chk & 255u) == 0u) {
      const bool over = global_ns() > deadline;
      if (__any_sync(kFull, over)) {
        if (!late && lane == 0) atomicOr(&args.stats->status, kErrWait);
        late = true;
        qdone = true;
      }
      if (args.tail_count && !late) {
        // the queue is used up and only the slowest few positions are left:
        // they go back to the host, which spreads each over the whole GPU
        unsigned rest = 0xFFFFFFFFu;
        if (lane == 0 && ld_global_volatile(&args.stats->next) >= n)
          rest = n - ld_global_volatile(&args.stats->done);
        rest = __shfl_sync(kFull, rest, 0);
        if (rest <= args.tail_count) {
          late = true;
          qdone = true;
          handoff = true;
          if (args.tail_bound && busy && !helper) {
            // what the root knows: its completed moves' best value (a lower
            // bound of its score), from its own registers or its frame
            int lb = -65;
            if (E == root_e) {
              if (!passed) lb = best;
            } else {
              u64 m0, f0;
              unsigned x0;
              fr.load(root_e, m0, f0, x0);
              if (!meta_passed(x0)) lb = meta_best(x0);
            }
            args.tail_bound[pos] = static_cast<signed char>(lb);
          }
        }
      }
    }
    if (late && busy) abort = true;
    // a helper whose split node was cut off abandons its subtree
    if (busy && helper && !abort && ld_shared_volatile(&sp.cut[wbase + towner])) abort = true;

    // ---- free lanes take input positions (at most rpw searches of its own
    //      per warp; the rest of the warp helps).  A warp holding a search
    //      that has run past hard_nodes takes no new positions: its lanes
    //      help that search as they come free (the other warps keep taking
    //      the queue), so the slowest positions get helpers early instead
    //      of finishing alone after the queue has run out. ----
    const unsigned own = __ballot_sync(kFull, busy && !helper);
    const bool hard = args.hard_nodes && __any_sync(kFull, busy && !helper && nodes > args.hard_nodes);
    if (!qdone) {
      const unsigned freem = __ballot_sync(kFull, !busy);
      const int quota = hard ? 0 : rpw - __popc(own);
      if (freem && quota > 0) {
        unsigned takers = freem;
        while (__popc(takers) > quota) takers &= ~(1u << (31 - __clz(static_cast<int>(takers))));
        const int leader = __ffs(static_cast<int>(takers)) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(&args.stats->next, static_cast<unsigned>(__popc(takers)));
        base = __shfl_sync(kFull, base, leader);
        if (base + static_cast<unsigned>(__popc(takers)) >= n) qdone = true;
        if ((takers >> lane) & 1u) {
          const unsigned k = base + static_cast<unsigned>(__popc(takers & lane_lt));
          if (k < n) {
            const unsigned p = args.perm[k];
            P = args.player[p];
            O = args.opp[p];
            E = 64 - popc(P | O);
            if ((P & O) || E > args.depth) {  // rejected input: flagged, not searched
              atomicOr(&args.stats->status, (P & O) ? kErrOverlap : kErrDepth);
              args.score[p] = 0;
              if (args.best) args.best[p] = kMoveNoneDev;
              atomicAdd(&args.stats->done, 1u);
            } else {
              busy = true;
              helper = false;
              pos = p;
              alpha = args.root_window ? args.root_window[2 * p] : -64;
              beta = args.root_window ? args.root_window[2 * p + 1] : 64;
              phase = PH_INIT;
              root_e = E;
              P0 = P;
              O0 = O;
              best = -65;
              passed = 0;
              nodes = 1;
              rootbest = kMoveNoneDev;
              abort = false;
              closed = false;
              tres = false;
            }
          }
        }
      }
    }

    // ---- choose this lane's op; close finished nodes ----
    int op = OP_NONE, sq = 0;
    bool stall = false;
    if (busy) {
      if (phase != PH_INIT) {
        int pops = 0;
        for (;;) {
          bool more;
          if (phase == PH_KEY) more = true;
          else if (phase == PH_LIST) more = list_peek(moves) != 0xFFF || (moves & kListOverflow);
          else more = moves != 0;
          const bool at_split = spe != 0 && spe == E;
          if (at_split) {  // fold in what the helpers found
            const unsigned a = ld_shared_volatile(&sp.acc[t]);
            if (a) {
              const int v = acc_value(a);
              if (v > best) {
                best = v;
                if (E == root_e && !passed) rootbest = static_cast<int>(a & 255u);
                if (v > alpha) alpha = v;
              }
            }
          }
          const bool fresh = best == -65;  // nothing searched yet
          const bool finished = abort || alpha >= beta || (!more && !fresh);
          if (!finished) {
            if (at_split) {
              const int lo = alpha > best ? alpha : best;
              if (lo > ld_shared_volatile(&sp.lo[t])) sp.lo[t] = lo;
            }
            break;
          }
          if (at_split) {
            if (ld_shared_volatile(&sp.pend[t]) != 0u) {  // helpers still out: wait for them
              if (abort || alpha >= beta) sp.cut[t] = 1u;
              stall = true;
              break;
            }
            const unsigned a = ld_shared_volatile(&sp.acc[t]);  // their last reports
            if (a && acc_value(a) > best) {
              best = acc_value(a);
              if (E == root_e && !passed) rootbest = static_cast<int>(a & 255u);
            }
            spe = 0;
          }
          // the node closes with value `best`
          // (after a pass, P / O / best / beta are those of the position
          // after the pass, which is the one recorded)
          if (!closed && !abort && args.tt_min && E >= args.tt_min)
            tt_updates += tt_record(args.tt, args.tt_bits, P, O, best, beta);
          closed = false;
          const int r = passed ? -best : best;
          if (E == root_e) {
            if (!helper) {  // the lane's own input position is solved
              if (args.nodes_out) atomicAdd(&args.nodes_out[pos], nodes);
              total_nodes += nodes;
              args.score[pos] = static_cast<signed char>(abort ? (handoff ? kUnsolvedDev : 0) : r);
              if (args.best) args.best[pos] = static_cast<signed char>(abort ? kMoveNoneDev : rootbest);
              atomicAdd(&args.stats->done, 1u);
              if (abort && handoff) atomicAdd(&args.stats->handed, 1u);
              busy = false;
              break;
            }
            const int v = -r;  // the value of the handed-out move for the split node
            const int o = wbase + towner;
            if (!abort && !tres && tlo + 1 < tbeta && v > tlo && v < tbeta &&
                !ld_shared_volatile(&sp.cut[o])) {
              // it beat the null window: search it again above what is known now
              int lo_now = ld_shared_volatile(&sp.lo[o]);
              const unsigned a = ld_shared_volatile(&sp.acc[o]);
              if (a && acc_value(a) > lo_now) lo_now = acc_value(a);
              const int a2 = v - 1 > lo_now ? v - 1 : lo_now;
              if (a2 < tbeta) {
                tres = true;
                tlo = a2;
                P = P0;
                O = O0;
                passed = 0;
                alpha = -tbeta;
                beta = -a2;
                best = -65;
                phase = PH_INIT;
                ++nodes;
                break;
              }
            }
            if (!abort) {
              const int exact = tres && v > tlo && v < tbeta;
              atomicMax(&sp.acc[o], pack_acc(v, exact, tsq));
            }
            if (args.nodes_out) atomicAdd(&args.nodes_out[pos], nodes);
            total_nodes += nodes;
            atomicSub(&sp.pend[o], 1u);
            busy = false;
            helper = false;
            break;
          }
          if (pops == kMaxPops) {  // more levels to return: next iteration
            stall = true;
            break;
          }
          ++pops;
          // back to the parent, unless this child must be searched again
          u64 m, f;
          unsigned meta;
          fr.load(E + 1, m, f, meta);
          const int pa = meta_alpha(meta), pb = meta_beta(meta), pbest = meta_best(meta);
          const int v = -r;
          const int plo = pa > pbest ? pa : pbest;
          if (passed) {  // back to the orientation the node was created in
            const u64 tmp = P;
            P = O;
            O = tmp;
          }
          if (!abort && !(f & kResearch) && pbest > -65 && plo + 1 < pb && v > plo && v < pb) {
            // the child beat its null window: search it again with the
            // window above its result (it is known to be worth at least v)
            *fr.f_ptr(E + 1) = f | kResearch;
            passed = 0;
            alpha = -pb;
            beta = 1 - v;
            best = -65;
            phase = PH_INIT;
            ++nodes;
            break;
          }
          ++E;
          moves = m;
          alpha = pa;
          beta = pb;
          best = pbest;
          passed = meta_passed(meta);
          phase = meta_list(meta) ? PH_LIST : PH_MASK;
          const int psq = meta_sq(meta);
          const u64 ff = f & ~kResearch;
          const u64 pP = O ^ ff ^ (1ULL << psq), pO = P ^ ff;
          P = pP;
          O = pO;
          if (v > best) {
            best = v;
            if (E == root_e && !passed) rootbest = psq;
            if (v > alpha) alpha = v;
          }
        }
      }
      if (busy && !stall) {
        if (phase == PH_INIT) {
          op = OP_INIT;
        } else if (phase == PH_KEY) {
          const u64 b = moves & (0ULL - moves);
          moves ^= b;
          sq = ctz64(b);
          op = OP_KEY;
        } else if (phase == PH_LIST) {
          const int e = list_peek(moves);
          if (e != 0xFFF) {
            sq = e & 63;
            moves += 1ULL << 60;  // next list index
            op = OP_MOVE;
          } else {
            op = OP_REMASK;
          }
        } else if (moves) {
          const u64 b = pick_parity(moves, ~(P | O));
          moves ^= b;
          sq = ctz64(b);
          op = OP_MOVE;
        } else {
          op = OP_PASS;  // no move and nothing searched: pass or game over
        }
      }
    }

    // ---- idle lanes take moves of split nodes of their warp ----
    u64 hX = 0, hY = 0;
    const unsigned freem = __ballot_sync(kFull, !busy);
    const bool can_help = args.help_min > 0 && (qdone || hard || __popc(own) >= rpw);
    if (freem && can_help) {
      // a busy lane without a split node looks for one now and then
      if (busy && !stall && spe == 0 && !abort && (chk & 7u) == 0u && root_e >= args.help_min)
        spe = find_split_node(fr, sp, t, P0, O0, root_e, E, args.help_min);
      // offers: lanes below their split node with a move left in its frame
      bool offer = false;
      u64 om = 0;
      unsigned ometa = 0;
      int olo = 0, obeta = 0;
      if (busy && !stall && !abort && spe != 0 && E < spe && !ld_shared_volatile(&sp.cut[t])) {
        u64 f;
        fr.load(spe, om, f, ometa);
        olo = ld_shared_volatile(&sp.lo[t]);
        const unsigned a = ld_shared_volatile(&sp.acc[t]);
        if (a && acc_value(a) > olo) olo = acc_value(a);
        obeta = sp.beta[t];
        offer = olo < obeta && (meta_list(ometa) ? list_peek(om) != 0xFFF : om != 0);
      }
      const unsigned offm = __ballot_sync(kFull, offer);
      if (offm) {
        const int pairs = min(__popc(freem), __popc(offm));
        int partner = lane, hsq = 0;
        u64 sPv = 0, sOv = 0;
        if (offer) {
          const int k = __popc(offm & lane_lt);
          if (k < pairs) {
            partner = nth_bit(freem, k);
            sPv = sp.P[t];
            sOv = sp.O[t];
            if (meta_list(ometa)) {
              hsq = list_peek(om) & 63;
              om += 1ULL << 60;
            } else {
              const u64 b = pick_parity(om, ~(sPv | sOv));
              om ^= b;
              hsq = ctz64(b);
            }
            *fr.m_ptr(spe) = om;
            atomicAdd(&sp.pend[t], 1u);
            ++handouts;
          }
        }
        if (!busy) {
          const int k = __popc(freem & lane_lt);
          if (k < pairs) partner = nth_bit(offm, k);
        }
        const int g_sq = __shfl_sync(kFull, hsq, partner);
        const int g_lo = __shfl_sync(kFull, olo, partner);
        const int g_beta = __shfl_sync(kFull, obeta, partner);
        const unsigned g_pos = __shfl_sync(kFull, pos, partner);
        const u64 g_P = __shfl_sync(kFull, sPv, partner);
        const u64 g_O = __shfl_sync(kFull, sOv, partner);
        if (!busy && partner != lane) {
          busy = true;
          helper = true;
          towner = partner;
          tsq = g_sq;
          tlo = g_lo;
          tbeta = g_beta;
          tres = false;
          pos = g_pos;
          hX = g_P;
          hY = g_O;
          sq = g_sq;
          op = OP_HAND;
        }
      }
    }

    if (qdone && !__any_sync(kFull, busy)) break;
    if (!__any_sync(kFull, op != OP_NONE)) {
      __nanosleep(100);  // every busy lane is waiting for helpers
      continue;
    }

    // ---- the uniform heavy step: one flip, then a mobility or flips ----
    const bool play = op == OP_MOVE || op == OP_KEY || op == OP_HAND;
    const bool same = op == OP_INIT || op == OP_REMASK;
    const bool fold = op == OP_MOVE && E == 2;   // child has one empty: score it now
    const bool last = op == OP_MOVE && E == 1;   // the move fills the board
    const bool needmob = op != OP_NONE && !fold && !last;
    const u64 X = op == OP_HAND ? hX : P;
    const u64 Y = op == OP_HAND ? hY : O;
    const u64 bit = play ? (1ULL << sq) : 0ULL;
    const u64 f = play ? gpo_flip(X, Y, sq, rays) : 0ULL;
    const u64 cP = same ? X : (Y ^ f);
    const u64 cO = same ? Y : (X ^ f ^ bit);
    int s1 = 0;
    if (__any_sync(kFull, fold)) {
      // the child (cP to move) has one empty square s: it plays s if it can,
      // else cO does, else the game ends with s empty
      const int s = ctz64(~(cP | cO)) & 63;  // & 63: lanes without a fold may hold none
      const int n1 = gpo_last_count(cP, s, lcnt, dmask);
      const int n2 = gpo_last_count(cO, s, lcnt, dmask);
      s1 = n1 ? 2 * (popc(cP) + n1 + 1) - 64
              : (n2 ? 64 - 2 * (popc(cO) + n2 + 1) : gpo_final(cP, cO));
    }
    u64 cm = 0;
    if (__any_sync(kFull, needmob)) cm = gpo_mobility(cP, cO);

    // ---- bookkeeping on the result ----
    // A node enters the keying phase (fastest-first) when it has two or more
    // moves and at least args.ff empties: `moves` then holds the squares
    // still to key and `lst` the list being built; the list replaces
    // `moves` when done.
    bool start_keys = false, created = false;
    if (op == OP_HAND) {  // a helper's root: the handed-out move's child
      P = cP;
      O = cO;
      E = 64 - popc(cP | cO);
      root_e = E;
      P0 = P;
      O0 = O;
      best = -65;
      passed = 0;
      nodes = 1;
      rootbest = kMoveNoneDev;
      abort = false;
      closed = false;
      alpha = -(tlo + 1);  // null window above the split node's bound
      beta = -tlo;
      moves = cm;
      phase = PH_MASK;
      start_keys = (cm & (cm - 1)) && E >= args.ff;
      created = true;
    } else if (op == OP_KEY) {
      int k = popc(cm) * 2 + ((bit & kCorners) ? 0 : 1);
      if (k > 62) k = 62;
      lst = list_insert(lst, k, sq);
      if (!moves) {
        moves = lst;
        phase = PH_LIST;
      }
    } else if (op == OP_INIT) {
      moves = cm;
      phase = PH_MASK;
      start_keys = (cm & (cm - 1)) && E >= args.ff;
      created = E == root_e && best == -65 && !helper;  // an input position's first init
    } else if (op == OP_REMASK) {
      moves = cm & ~list_squares(moves);
      phase = PH_MASK;
    } else if (op == OP_PASS) {
      ++nodes;
      if (!cm) {  // neither side can move: the game is over
        best = gpo_final(P, O);
        moves = 0;
        if (E == root_e) rootbest = kMoveNoneDev;
      } else {
        P = cP;
        O = cO;
        const int a = alpha;
        alpha = -beta;
        beta = -a;
        passed = 1;
        moves = cm;
        phase = PH_MASK;
        start_keys = (cm & (cm - 1)) && E >= args.ff;
        if (E == root_e) rootbest = kMovePassDev;
        // the position after the pass is a node of its own: it gets the table
        // probe and the stability cutoff (positions where one side keeps
        // passing are the lopsided ones, whose searches are the longest)
        created = true;
      }
    } else if (op == OP_MOVE) {
      ++nodes;
      if (last || fold) {
        const int v = last ? -gpo_final(cP, cO) : -s1;
        if (v > best) {
          best = v;
          if (E == root_e && !passed) rootbest = sq;
          if (v > alpha) alpha = v;
        }
      } else {
        const int lo = alpha > best ? alpha : best;
        fr.store(E, moves, f, pack_meta(sq, alpha, beta, best, passed, phase == PH_LIST));
        // first move: the node's window; later moves: a null window above lo
        const int na = (best > -65 && lo + 1 < beta) ? -(lo + 1) : -beta;
        --E;
        P = cP;
        O = cO;
        alpha = na;
        beta = -lo;
        best = -65;
        passed = 0;
        moves = cm;
        phase = PH_MASK;
        start_keys = (cm & (cm - 1)) && E >= args.ff;
        created = true;
      }
    }
    if (created && !abort && op != OP_INIT) {
      if (args.tt_min && E >= args.tt_min) {
        ++tt_probes;
        const unsigned h = tt_lookup(args.tt, args.tt_bits, P, O);
        if (h) {
          ++tt_hits;
          const int lb = static_cast<int>((h >> 8) & 0xff) - 64, ub = static_cast<int>(h & 0xff) - 64;
          // a bound outside the window closes the node at once; one
          // inside narrows it (sound for fail-soft search)
          if (lb >= beta || ub <= alpha || lb >= ub) {
            best = lb >= beta ? lb : (ub <= alpha ? ub : lb);
            alpha = beta;
            closed = true;
            start_keys = false;
          } else {
            if (lb > alpha) alpha = lb;
            if (ub < beta) beta = ub;
          }
        }
      }
      // the cutoff needs about (64 - alpha) / 2 stable discs; few empties leave
      // many stable discs, so the alpha it is worth checking at rises with E
      if (!closed && args.stab_min && E >= args.stab_min && alpha >= args.stab_gate + 3 * E) {
        const int cap = 64 - 2 * stable_count(O, P | O);
        if (cap <= alpha) {  // the side to move cannot reach alpha
          best = cap;
          alpha = beta;
          closed = true;
          start_keys = false;
          ++stab_cuts;
        }
      }
      if (args.node_budget && nodes > args.node_budget && !helper) {
        // watchdog: every open node of this lane closes at once; the call
        // reports the error
        atomicOr(&args.stats->status, kErrBudget);
        abort = true;
      }
    }
    if (created && !closed && args.order_table && E >= args.learned_min && (cm & (cm - 1))) {
      const u64 l = order_lookup(args.order_table, args.order_bits, P, O);
      if (l) {  // the learned orderer's five best moves replace the ordering probes
        moves = l;
        phase = PH_LIST;
        start_keys = false;
      }
    }
    if (start_keys) {
      phase = PH_KEY;
      lst = kListEmpty;
    }
  }
  warp_add(&args.stats->nodes, total_nodes);
  warp_add(&args.stats->handouts, handouts);
  warp_add(&args.stats->stab_cuts, stab_cuts);
  warp_add(&args.stats->tt_probes, tt_probes);
  warp_add(&args.stats->tt_hits, tt_hits);
  warp_add(&args.stats->tt_updates, tt_updates);
}

size_t batched_smem_bytes(int threads, int smem_top) {
  const int sslots = smem_top >= 3 ? smem_top - 2 : 0;
  return kTableBytes + static_cast<size_t>(threads) * (kSplitBytes + sslots * kFrameBytes);
}

cudaError_t batched_grid(int threads, int smem_top, int sms, int* grid, size_t* smem) {
  *smem = batched_smem_bytes(threads, smem_top);
  cudaError_t e = cudaFuncSetAttribute(batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(*smem));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_kernel, threads, *smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  *grid = per_sm * sms;
  return cudaSuccess;
}

cudaError_t batched_plan(int threads, int depth, int* smem_top) {
  // Blocks per SM that registers allow; the frames go to shared memory when
  // all depth - 2 slots fit beside that many blocks, else to global memory.
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_kernel, threads, 0);
  if (e != cudaSuccess) return e;
  int dev = 0, smem_sm = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  // 1 KB per block is reserved by the hardware
  const long per_block = static_cast<long>(smem_sm) / per_sm - 1024 - kTableBytes -
                         static_cast<long>(threads) * kSplitBytes;
  const long need = static_cast<long>(depth > 2 ? depth - 2 : 0) * threads * kFrameBytes;
  *smem_top = need <= per_block ? depth : 2;
  return cudaSuccess;
}

size_t batched_gframe_bytes(int depth, int smem_top, size_t lanes) {
  if (depth <= smem_top) return 0;
  return static_cast<size_t>(depth > 2 ? depth - 2 : 0) * kFrameBytes * lanes;
}

cudaError_t launch_batched_shape(const BatchedArgs& args, int grid, int threads, size_t smem,
                                 cudaStream_t s) {
  batched_kernel<<<grid, threads, smem, s>>>(args);
  return cudaGetLastError();
}

cudaError_t launch_batched(const BatchedArgs& args, BatchedLaunch& cfg, int sms, cudaStream_t s) {
  const int threads = cfg.threads > 0 ? cfg.threads : 128;
  int grid = 0;
  size_t smem = 0;
  cudaError_t e = batched_grid(threads, args.smem_top, sms, &grid, &smem);
  if (e != cudaSuccess) return e;
  if (cfg.grid > 0 && cfg.grid < grid) grid = cfg.grid;
  cfg.grid = grid;
  cfg.smem = smem;
  // Lanes wait only for lanes of their own warp, so an ordinary launch
  // suffices: warps leave as soon as the queue is used up and their lanes
  // are idle.
  batched_kernel<<<grid, threads, smem, s>>>(args);
  return cudaGetLastError();
}

}  // namespace gpo
