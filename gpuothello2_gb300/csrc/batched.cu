// Batched solver: one persistent launch over a device work queue of
// positions ordered by empty count (most empties first); one lane searches
// one position at a time and refills itself from the queue when done.
//
// Uniform-step engine.  Thread-per-board search diverges because lanes sit
// at different kinds of nodes.  Here every loop iteration does the same
// heavy work in every lane -- one flip and one mobility:
//
//   op INIT    mobility of a new root
//   op MOVE    play square sq: flip, child position, child mobility; the
//              child is pushed (or scored at once when it fills the board)
//   op PASS    the side to move has no move: child = swapped position and
//              its mobility (no mobility there either = game over)
//   op KEY     ordering probe at a fastest-first node: the opponent's
//              mobility after square sq becomes that move's sort key
//   op REMASK  mobility of the current node again, to search the moves that
//              did not fit in its five-entry ordered list
//
// and only cheap bookkeeping diverges: choosing the op, returning finished
// nodes to their parents (a short loop of frame pops), inserting keys.
//
// Search (values identical to the reference's negamax, tree different):
// fail-soft alpha-beta; nodes with >= ff empties search their moves in
// fastest-first order (fewest opponent replies, corners first on ties), the
// role of the reference's sorted UpperNode list (solver.cu:78-93); nodes
// below ff use corner/parity order from the move mask.  Passes happen in
// place with the window negated and swapped (solver.cu:57-73, 214-221,
// 246-256 semantics).
//
// Frames: a node with E empties saves {move word, flips of the move being
// searched, packed alpha/beta/best/square/flags} in slot E when it pushes a
// child.  The move word is the remaining-move mask, or at fastest-first
// nodes the packed ordered list (search.cuh), so no per-thread local memory
// is used.  Slots 2..smem_top are in shared memory, interleaved by thread
// ([slot][thread]: a warp touches 32 consecutive words); the rarely touched
// slots above smem_top are in a per-lane global array (L2-resident).
#include "common.cuh"
#include "kernels.h"
#include "search.cuh"
#include "table.cuh"

namespace gpo {

namespace {

enum : int { OP_NONE = 0, OP_INIT, OP_MOVE, OP_PASS, OP_KEY, OP_REMASK, OP_DONATE };
enum : int { PH_INIT = 0, PH_MASK, PH_KEY, PH_LIST };

constexpr int kFrameBytes = 20;
constexpr int kRayBytes = 256 * 8;

__device__ __forceinline__ unsigned pack_meta(int sq, int alpha, int beta, int best, int passed,
                                              int list) {
  return static_cast<unsigned>(sq) | (static_cast<unsigned>(alpha & 0xff) << 6) |
         (static_cast<unsigned>(beta & 0xff) << 14) | (static_cast<unsigned>(best & 0xff) << 22) |
         (static_cast<unsigned>(passed) << 30) | (static_cast<unsigned>(list) << 31);
}

struct Frames {
  u64* sM;
  u64* sF;
  unsigned* sX;
  u64* gM;
  u64* gF;
  unsigned* gX;
  int B, t, top;
  size_t G, gid;

  __device__ __forceinline__ void store(int E, u64 m, u64 f, unsigned x) const {
    if (E <= top) {
      const int i = (E - 2) * B + t;
      sM[i] = m;
      sF[i] = f;
      sX[i] = x;
    } else {
      const size_t i = static_cast<size_t>(E - top - 1) * G + gid;
      gM[i] = m;
      gF[i] = f;
      gX[i] = x;
    }
  }
  __device__ __forceinline__ void load(int E, u64& m, u64& f, unsigned& x) const {
    if (E <= top) {
      const int i = (E - 2) * B + t;
      m = sM[i];
      f = sF[i];
      x = sX[i];
    } else {
      const size_t i = static_cast<size_t>(E - top - 1) * G + gid;
      m = gM[i];
      f = gF[i];
      x = gX[i];
    }
  }
};

}  // namespace

__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) {
  return *reinterpret_cast<const volatile unsigned*>(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
#ifdef GPO_SIMT_EMU  // the CPU emulation of this kernel used by the tests
  return gpo_emu_ns();
#else
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
#endif
}

__device__ __forceinline__ unsigned pack_result(int v, int move) {
  return (static_cast<unsigned>(v + 128) << 8) | static_cast<unsigned>(move & 255);
}

__global__ void __launch_bounds__(256) batched_kernel(BatchedArgs args) {
  extern __shared__ __align__(16) u64 smem_raw[];
  u64* const rays = smem_raw;           // 64 x 4 up-ray table (bitboard.cuh)
  u64* const smem_u64 = smem_raw + 256;  // frame slots
  gpo_build_rays(rays);
  __syncthreads();
  Frames fr;
  fr.B = blockDim.x;
  fr.t = threadIdx.x;
  fr.top = args.smem_top;
  const int sslots = args.smem_top >= 2 ? args.smem_top - 1 : 0;
  fr.sM = smem_u64;
  fr.sF = smem_u64 + sslots * fr.B;
  fr.sX = reinterpret_cast<unsigned*>(smem_u64 + 2 * sslots * fr.B);
  fr.G = static_cast<size_t>(gridDim.x) * blockDim.x;
  fr.gid = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int gslots = args.depth > args.smem_top ? args.depth - args.smem_top : 0;
  fr.gM = reinterpret_cast<u64*>(args.gframes);
  fr.gF = fr.gM + gslots * fr.G;
  fr.gX = reinterpret_cast<unsigned*>(fr.gF + gslots * fr.G);
  const size_t G = fr.G, gid = fr.gid;

  const unsigned lane = threadIdx.x & 31;
  const unsigned lane_lt = (1u << lane) - 1u;
  const unsigned n = static_cast<unsigned>(args.n);
  constexpr unsigned kNoMbox = 0xFFFFFFFFu;
  unsigned long long total_nodes = 0, donations = 0, cancels = 0;
  unsigned long long tt_probes = 0, tt_hits = 0, tt_updates = 0;
  bool tt_cut = false;  // the current node was closed by a table bound when created

  // abort: close every open node of this lane's root at once (node budget
  // exceeded, or the subtree was cancelled by its donor); an aborted
  // subtree reports nothing but its completion.
  bool busy = false, waiting = false, exhausted = false, started = false, abort = false;
  unsigned pos = 0, task_mbox = kNoMbox, qidx = 0, chk = 0, dmask = 0;
  int task_sq = 0;
  // One deadline for the whole launch bounds every wait: a lane holding a
  // ticket never gives it up early (a donor may still fill it), and when
  // the deadline passes every lane unwinds and the call reports an error.
  const unsigned long long deadline = global_ns() + args.wait_limit_ns;
  bool late = false;
  u64 P = 0, O = 0, moves = 0, lst = 0, P0 = 0, O0 = 0;
  int alpha = 0, beta = 0, best = 0, passed = 0, E = 0, root_e = 0, phase = PH_INIT;
  int rootbest = kMoveNoneDev;
  unsigned long long nodes = 0;

  for (;;) {
    // ---- lanes without work: a queued subtree first (hard positions split
    //      early must not wait behind the input queue) ----
    if (!busy && !waiting && !exhausted && args.donate_min > 0) {
      const unsigned h = ld_volatile(&args.stats->dq_head);
      if (h < ld_volatile(&args.stats->dq_tail) && atomicCAS(&args.stats->dq_head, h, h + 1u) == h) {
        qidx = h;
        waiting = true;
      }
    }
    // ---- then the input queue (one atomic per warp) ----
    const unsigned need = __ballot_sync(0xffffffffu, !busy && !waiting && !exhausted);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned base = 0;
      if (static_cast<int>(lane) == leader) base = atomicAdd(&args.stats->next, __popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!busy && !waiting && !exhausted) {
        const unsigned k = base + __popc(need & lane_lt);
        if (k < n) {
          const unsigned p = args.perm[k];
          P = args.player[p];
          O = args.opp[p];
          E = 64 - popc(P | O);
          if ((P & O) || E > args.depth) {  // rejected input: flagged, not searched
            atomicOr(&args.stats->status, (P & O) ? kErrOverlap : kErrDepth);
            args.score[p] = 0;
            if (args.best) args.best[p] = kMoveNoneDev;
            __threadfence();
            atomicAdd(&args.stats->done, 1u);
          } else {
            busy = started = true;
            pos = p;
            task_mbox = kNoMbox;
            alpha = args.root_alpha ? args.root_alpha[p] : -64;
            beta = args.root_beta ? args.root_beta[p] : 64;
          }
        } else if (args.donate_min > 0) {
          qidx = atomicAdd(&args.stats->dq_head, 1u);  // wait for a donated subtree
          waiting = true;
        } else {
          exhausted = true;
        }
      }
    }
    if (waiting) {
      const unsigned qslot = qidx % args.task_cap;
      if (ld_volatile(&args.ready[qslot]) == qidx + 1u) {
        // The record was written by another SM: read it from L2 (.cg),
        // never from a possibly stale L1 line.
        __threadfence();
        const DonatedTask* q = args.queue + qslot;
        P = __ldcg(&q->player);
        O = __ldcg(&q->opp);
        const unsigned w = __ldcg(&q->window);
        task_mbox = __ldcg(&q->mbox);
        pos = __ldcg(&q->top);
        __threadfence();
        atomicExch(&args.consumed[qslot], qidx + 1u);  // the record may be refilled
        E = 64 - popc(P | O);
        alpha = static_cast<signed char>(w & 0xff);
        beta = static_cast<signed char>((w >> 8) & 0xff);
        task_sq = static_cast<int>((w >> 16) & 0xff);
        waiting = false;
        busy = started = true;
      } else if (ld_volatile(&args.stats->done) >= n) {
        waiting = false;
        exhausted = true;
      } else if (global_ns() > deadline) {
        atomicOr(&args.stats->status, kErrWait);
        waiting = false;
        exhausted = true;
      }
    }
    if (started) {  // a position or subtree was just taken: it is this lane's root
      started = false;
      phase = PH_INIT;
      root_e = E;
      P0 = P;
      O0 = O;
      best = -65;
      passed = 0;
      nodes = 1;
      rootbest = kMoveNoneDev;
      dmask = 0;
      abort = false;
    }
    if (__ballot_sync(0xffffffffu, !exhausted) == 0) break;

    // ---- choose this lane's op; return finished nodes to their parents ----
    int op = OP_NONE, sq = 0;
    u64 DX = 0, DY = 0;
    unsigned dq = 0, dwin = 0, dmbox = 0;
    if (busy) {
      if (phase == PH_INIT) {
        op = OP_INIT;
      } else {
        bool stall = false;
        for (;;) {
          bool more;
          if (phase == PH_KEY) more = true;
          else if (phase == PH_LIST) more = list_peek(moves) != 0xFFF || (moves & kListOverflow);
          else more = moves != 0;
          const bool fresh = best == -65;  // nothing searched yet
          const bool finished = abort || alpha >= beta || (!more && !fresh);
          if (!finished) break;
          if ((dmask >> E) & 1u) {
            // moves handed to other lanes must report before the node closes;
            // after a cutoff (or an abort) their results no longer matter
            const size_t mb = static_cast<size_t>(E) * G + gid;
            if (ld_volatile(&args.mbox_pend[mb]) != 0u) {
              bool cut = abort || alpha >= beta;
              if (!cut) {
                const unsigned a = ld_volatile(&args.mbox_acc[mb]);
                cut = a && static_cast<int>(a >> 8) - 128 >= beta;
              }
              if (cut && !ld_volatile(&args.mbox_cancel[mb])) {
                atomicExch(&args.mbox_cancel[mb], 1u);
                ++cancels;
              }
              if (!late && global_ns() <= deadline) {
                stall = true;
                break;
              }
              late = true;
              atomicOr(&args.stats->status, kErrWait);
            }
            __threadfence();
            const unsigned a = atomicAdd(&args.mbox_acc[mb], 0u);
            if (a) {
              const int v = static_cast<int>(a >> 8) - 128;
              if (v > best) {
                best = v;
                if (E == root_e && !passed) rootbest = static_cast<int>(a & 255u);
                if (v > alpha) alpha = v;
              }
            }
            dmask &= ~(1u << E);
          }
          if (tt_cut) {
            tt_cut = false;
          } else if (args.tt_min && E >= args.tt_min && !passed && !abort) {
            // best >= beta proves value >= best; anything lower proves
            // value <= best (an exact value is also an upper bound)
            const TTKey k = tt_key(P, O);
            const bool ok = best >= beta ? tt_store(args.tt, args.tt_bits, k, best, 64)
                                         : tt_store(args.tt, args.tt_bits, k, -64, best);
            tt_updates += ok;
          }
          const int r = passed ? -best : best;
          if (E == root_e) {  // the lane's root is done
            if (args.nodes_out) atomicAdd(&args.nodes_out[pos], nodes);
            total_nodes += nodes;
            if (task_mbox == kNoMbox) {
              args.score[pos] = static_cast<signed char>(abort ? (args.budget_mark ? -128 : 0) : r);
              if (args.best) args.best[pos] = static_cast<signed char>(rootbest);
              __threadfence();
              atomicAdd(&args.stats->done, 1u);
            } else {
              if (!abort) atomicMax(&args.mbox_acc[task_mbox], pack_result(-r, task_sq));
              __threadfence();
              atomicSub(&args.mbox_pend[task_mbox], 1u);
              atomicSub(&args.pos_tasks[pos], 1u);
            }
            busy = false;
            break;
          }
          if (passed) {  // back to the orientation the node was created in
            const u64 tmp = P;
            P = O;
            O = tmp;
          }
          ++E;
          u64 f;
          unsigned meta;
          fr.load(E, moves, f, meta);
          const int psq = static_cast<int>(meta & 63u);
          alpha = static_cast<signed char>((meta >> 6) & 0xff);
          beta = static_cast<signed char>((meta >> 14) & 0xff);
          best = static_cast<signed char>((meta >> 22) & 0xff);
          passed = static_cast<int>((meta >> 30) & 1u);
          phase = (meta >> 31) ? PH_LIST : PH_MASK;
          const u64 bit = 1ULL << psq;
          const u64 pP = O ^ f ^ bit, pO = P ^ f;
          P = pP;
          O = pO;
          const int v = -r;
          if (v > best) {
            best = v;
            if (E == root_e && !passed) rootbest = psq;
            if (v > alpha) alpha = v;
          }
        }
        // ---- a handed-out subtree whose donor was cut off stops early ----
        ++chk;
        if (busy && !abort && task_mbox != kNoMbox && (chk & 15u) == 0u &&
            ld_volatile(&args.mbox_cancel[task_mbox]))
          abort = true;
        if (busy && !abort && (chk & 255u) == 0u && global_ns() > deadline) {
          atomicOr(&args.stats->status, kErrWait);
          late = abort = true;
        }
        // ---- donation: hand a move of an ancestor to a waiting lane ----
        if (busy && !stall && !abort && E < root_e && args.donate_min > 0 &&
            root_e >= args.donate_min && (chk & 15u) == 8u) {
          const unsigned t = ld_volatile(&args.stats->dq_tail);
          const unsigned h = ld_volatile(&args.stats->dq_head);
          // Hand out a move when a lane waits for one (ticket t is held), or
          // when this root has run long (a hard position: split it while
          // the rest of the batch still keeps the GPU busy) and few records
          // are queued; record t % cap must have been read by the holder of
          // ticket t - cap.
          const bool asked = t < h;
          const bool pushed = !asked && nodes > args.long_nodes && t - h < 1024u;
          if ((asked || pushed) && ld_volatile(&args.pos_tasks[pos]) < args.max_tasks &&
              (t < args.task_cap ||
               ld_volatile(&args.consumed[t % args.task_cap]) == t - args.task_cap + 1u)) {
            // Walk the path from the root (replaying the stored flips) to the
            // shallowest node whose first move has returned and that has an
            // untried move.
            u64 X = P0, Y = O0;
            int de = -1;
            u64 dm = 0, df = 0;
            unsigned dmeta = 0;
            int dlo = 0, db = 0;
            for (int e = root_e; e > E; --e) {
              u64 m, f;
              unsigned meta;
              fr.load(e, m, f, meta);
              const int pas = static_cast<int>((meta >> 30) & 1u);
              if (pas) {
                const u64 tmp = X;
                X = Y;
                Y = tmp;
              }
              const int b0 = static_cast<signed char>((meta >> 14) & 0xff);
              const int best0 = static_cast<signed char>((meta >> 22) & 0xff);
              if (e >= args.donate_min && !pas && best0 > -65) {
                const int a0 = static_cast<signed char>((meta >> 6) & 0xff);
                int lo0 = a0 > best0 ? a0 : best0;
                if ((dmask >> e) & 1u) {
                  const unsigned a = ld_volatile(&args.mbox_acc[static_cast<size_t>(e) * G + gid]);
                  if (a && static_cast<int>(a >> 8) - 128 > lo0) lo0 = static_cast<int>(a >> 8) - 128;
                }
                if (lo0 < b0) {
                  if (meta >> 31) {
                    const int en = list_peek(m);
                    if (en != 0xFFF) {
                      sq = en & 63;
                      dm = m + (1ULL << 60);
                      de = e;
                    }
                  } else if (m) {
                    const u64 b = pick_parity(m, ~(X | Y));
                    sq = ctz64(b);
                    dm = m ^ b;
                    de = e;
                  }
                  if (de >= 0) {
                    df = f;
                    dmeta = meta;
                    dlo = lo0;
                    db = b0;
                    break;
                  }
                }
              }
              const u64 bit = 1ULL << (meta & 63u);
              const u64 cx = Y ^ f, cy = X ^ f ^ bit;
              X = cx;
              Y = cy;
            }
            if (de >= 0 && atomicCAS(&args.stats->dq_tail, t, t + 1u) == t) {
              fr.store(de, dm, df, dmeta);
              const size_t mb = static_cast<size_t>(de) * G + gid;
              if (!((dmask >> de) & 1u)) {
                atomicExch(&args.mbox_acc[mb], 0u);
                atomicExch(&args.mbox_pend[mb], 0u);
                atomicExch(&args.mbox_cancel[mb], 0u);
                dmask |= 1u << de;
              }
              atomicAdd(&args.mbox_pend[mb], 1u);
              atomicAdd(&args.pos_tasks[pos], 1u);
              op = OP_DONATE;
              DX = X;
              DY = Y;
              dq = t;
              dmbox = static_cast<unsigned>(mb);
              dwin = static_cast<unsigned>((-db) & 0xff) | (static_cast<unsigned>((-dlo) & 0xff) << 8) |
                     (static_cast<unsigned>(sq) << 16);
            }
          }
        }
        if (busy && !stall && op == OP_NONE) {
          if (phase == PH_KEY) {
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
    }
    if (!__any_sync(0xffffffffu, op != OP_NONE)) {
      __nanosleep(200);  // idle or waiting warp: leave issue slots to busy warps
      continue;
    }

    // ---- the uniform heavy step: one flip, one mobility ----
    const bool play = op == OP_MOVE || op == OP_KEY || op == OP_DONATE;
    const bool same = op == OP_INIT || op == OP_REMASK;
    const u64 X = op == OP_DONATE ? DX : P;
    const u64 Y = op == OP_DONATE ? DY : O;
    const u64 bit = play ? (1ULL << sq) : 0ULL;
    const u64 f = play ? gpo_flip(X, Y, sq, rays) : 0ULL;
    const u64 cP = same ? X : (Y ^ f);
    const u64 cO = same ? Y : (X ^ f ^ bit);
    const u64 cm = gpo_mobility(cP, cO);

    // ---- bookkeeping on the result ----
    // A node enters the keying phase (fastest-first) when it has moves and
    // at least args.ff empties: `moves` then holds the squares still to key
    // and `lst` the list being built; the list replaces `moves` when done.
    bool start_keys = false;
    if (op == OP_DONATE) {
      const unsigned qslot = dq % args.task_cap;
      DonatedTask* q = args.queue + qslot;
      q->player = cP;
      q->opp = cO;
      q->window = dwin;
      q->mbox = dmbox;
      q->top = pos;
      q->pad = 0;
      __threadfence();
      atomicExch(&args.ready[qslot], dq + 1u);
      ++donations;
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
      start_keys = cm && E >= args.ff;
      if (cm && args.root_lists && task_mbox == kNoMbox && E >= args.learned_min) {
        moves = args.root_lists[pos];  // the learned orderer's five best moves
        phase = PH_LIST;
        start_keys = false;
      }
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
        start_keys = E >= args.ff;
        if (E == root_e) rootbest = kMovePassDev;
      }
    } else if (op == OP_MOVE) {
      ++nodes;
      const int lo = alpha > best ? alpha : best;
      if (E == 1) {  // the move fills the board
        const int v = -gpo_final(cP, cO);
        if (v > best) {
          best = v;
          if (E == root_e && !passed) rootbest = sq;
          if (v > alpha) alpha = v;
        }
      } else {
        fr.store(E, moves, f, pack_meta(sq, alpha, beta, best, passed, phase == PH_LIST));
        --E;
        P = cP;
        O = cO;
        alpha = -beta;
        beta = -lo;
        best = -65;
        passed = 0;
        moves = cm;
        phase = PH_MASK;
        start_keys = cm && E >= args.ff;
        if (args.tt_min && E >= args.tt_min && !abort) {
          int lb, ub;
          ++tt_probes;
          if (tt_probe(args.tt, args.tt_bits, tt_key(P, O), lb, ub)) {
            ++tt_hits;
            // a bound outside the window closes the node at once; one
            // inside narrows it (sound for fail-soft search)
            if (lb >= beta || ub <= alpha || lb >= ub) {
              best = lb >= beta ? lb : (ub <= alpha ? ub : lb);
              alpha = beta;
              tt_cut = true;
              start_keys = false;
            } else {
              if (lb > alpha) alpha = lb;
              if (ub < beta) beta = ub;
            }
          }
        }
        if (args.node_budget && nodes > args.node_budget && !abort) {
          // watchdog: every open node of this lane closes at once (still
          // collecting any handed-out moves); the call reports the error,
          // or, in a first pass, the position is marked for the second
          if (!args.budget_mark) atomicOr(&args.stats->status, kErrBudget);
          abort = true;
        }
      }
    }
    if (start_keys) {
      phase = PH_KEY;
      lst = kListEmpty;
    }
  }
  warp_add(&args.stats->nodes, total_nodes);
  warp_add(&args.stats->donations, donations);
  warp_add(&args.stats->cancels, cancels);
  warp_add(&args.stats->tt_probes, tt_probes);
  warp_add(&args.stats->tt_hits, tt_hits);
  warp_add(&args.stats->tt_updates, tt_updates);
}

cudaError_t batched_grid(int threads, int smem_top, int sms, int* grid, size_t* smem) {
  const int sslots = smem_top >= 2 ? smem_top - 1 : 0;
  *smem = kRayBytes + static_cast<size_t>(threads) * sslots * kFrameBytes;
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
  // Blocks per SM that registers allow, then as many shared-memory frame
  // slots as fit beside them without lowering that count.
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_kernel, threads, 0);
  if (e != cudaSuccess) return e;
  int dev = 0, smem_sm = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const int per_block = smem_sm / per_sm - 1024 - kRayBytes;  // 1 KB per block is reserved
  const int slots = per_block > 0 ? per_block / (threads * kFrameBytes) : 0;
  int top = slots + 1;
  if (top > depth) top = depth;
  if (top < 1) top = 1;
  *smem_top = top;
  return cudaSuccess;
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
  // Idle lanes wait (bounded) for subtrees donated by other blocks, so every
  // block must be resident at once: a cooperative launch guarantees it.
  BatchedArgs a = args;
  void* kargs[] = {&a};
  return cudaLaunchCooperativeKernel(reinterpret_cast<void*>(batched_kernel), dim3(grid),
                                     dim3(threads), kargs, smem, s);
}

}  // namespace gpo
