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

namespace gpo {

namespace {

enum : int { OP_NONE = 0, OP_INIT, OP_MOVE, OP_PASS, OP_KEY, OP_REMASK, OP_DONATE };
enum : int { PH_INIT = 0, PH_MASK, PH_KEY, PH_LIST };

constexpr int kFrameBytes = 20;

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

// Returns a finished task's value to its parent slot, walking up while this
// lane is the last one holding the parent open; writes the input position's
// score and best move at the top.  Every slot's accumulator holds the max
// of its children's fail-soft candidates packed with the move that made
// them; each candidate is either exact or a bound not above the true value
// (its window's lower edge was a value already proven), so the max is the
// node's fail-soft value and its move an optimal move.
__device__ __forceinline__ void finish_slot(const BatchedArgs& a, unsigned slot) {
  for (int guard = 0; guard < 2 * kMaxEmpties + 2; ++guard) {
    __threadfence();
    const unsigned packed = atomicAdd(&a.acc[slot], 0u);
    const int v = static_cast<int>(packed >> 8) - 128;
    if (slot < static_cast<unsigned>(a.n)) {
      a.score[slot] = static_cast<signed char>(v);
      if (a.best) a.best[slot] = static_cast<signed char>(packed & 255u);
      __threadfence();
      atomicAdd(&a.stats->done, 1u);
      return;
    }
    const unsigned i = slot - static_cast<unsigned>(a.n);
    const unsigned par = __ldcg(&a.parent[i]);
    const unsigned msq = __ldcg(&a.psq[i]);
    atomicMax(&a.acc[par], (static_cast<unsigned>(128 - v) << 8) | msq);
    __threadfence();
    if (atomicSub(&a.pending[par], 1u) != 1u) return;
    slot = par;
  }
  atomicOr(&a.stats->status, kErrInternal);
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  return *reinterpret_cast<const volatile unsigned*>(p);
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__global__ void __launch_bounds__(256) batched_kernel(BatchedArgs args) {
  extern __shared__ u64 smem_u64[];
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

  const unsigned lane = threadIdx.x & 31;
  const unsigned lane_lt = (1u << lane) - 1u;
  const unsigned n = static_cast<unsigned>(args.n);
  unsigned long long total_nodes = 0, donations = 0;

  bool busy = false, waiting = false, exhausted = false, started = false;
  unsigned slot = 0, top = 0, qidx = 0, chk = 0, dq = 0;
  unsigned long long wait_start = 0;
  u64 P = 0, O = 0, moves = 0, lst = 0, P0 = 0, O0 = 0;
  int alpha = 0, beta = 0, best = 0, passed = 0, E = 0, root_e = 0, phase = PH_INIT;
  int rootbest = kMoveNoneDev;
  unsigned long long nodes = 0;

  for (;;) {
    // ---- lanes without work: input queue first (one atomic per warp) ----
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
            busy = true;
            started = true;
            slot = p;
            top = p;
            alpha = -64;
            beta = 64;
            atomicExch(&args.acc[slot], 0u);
            atomicExch(&args.pending[slot], 1u);
          }
        } else if (args.donate_min > 0) {
          // nothing left to start: reserve the next donated task
          qidx = atomicAdd(&args.stats->dq_head, 1u);
          waiting = true;
          wait_start = global_ns();
        } else {
          exhausted = true;
        }
      }
    }
    if (waiting) {
      if (qidx < args.task_cap && ld_acquire(&args.ready[qidx])) {
        // Records and their side arrays were written by other SMs: read
        // them from L2 (ld.global.cg), never from a possibly stale L1 line.
        __threadfence();
        const DonatedTask* q = args.queue + qidx;
        waiting = false;
        busy = true;
        started = true;
        P = __ldcg(&q->player);
        O = __ldcg(&q->opp);
        E = 64 - popc(P | O);
        alpha = __ldcg(&q->alpha);
        beta = __ldcg(&q->beta);
        slot = __ldcg(&q->slot);
        top = __ldcg(&args.top[slot - n]);
      } else if (ld_acquire(&args.stats->done) >= n) {
        waiting = false;
        exhausted = true;
      } else if (global_ns() - wait_start > args.wait_limit_ns) {
        atomicOr(&args.stats->status, kErrWait);
        waiting = false;
        exhausted = true;
      }
    }
    if (started) {  // a task was just taken: its root is this lane's level 0
      started = false;
      phase = PH_INIT;
      root_e = E;
      P0 = P;
      O0 = O;
      best = -65;
      passed = 0;
      nodes = 1;
      rootbest = kMoveNoneDev;
    }
    const unsigned active = __ballot_sync(0xffffffffu, !exhausted);
    if (active == 0) break;
    if (__ballot_sync(0xffffffffu, busy) == 0) {
      __nanosleep(256);  // a warp of waiting lanes leaves issue slots to busy warps
      continue;
    }

    // ---- choose this lane's op; return finished nodes to their parents ----
    int op = OP_NONE, sq = 0;
    int dalpha = 0, dbeta = 0;
    if (busy) {
      if (phase == PH_INIT) {
        op = OP_INIT;
      } else {
        for (;;) {
          bool more;
          if (phase == PH_KEY) more = true;
          else if (phase == PH_LIST) more = list_peek(moves) != 0xFFF || (moves & kListOverflow);
          else more = moves != 0;
          const bool fresh = best == -65;  // nothing searched yet
          const bool finished = alpha >= beta || (!more && !fresh);
          if (!finished) break;
          const int r = passed ? -best : best;
          if (E == root_e) {  // this lane's part of the task is done
            if (args.nodes_out) atomicAdd(&args.nodes_out[top], nodes);
            total_nodes += nodes;
            atomicMax(&args.acc[slot], (static_cast<unsigned>(r + 128) << 8) |
                                           static_cast<unsigned>(rootbest));
            __threadfence();
            if (atomicSub(&args.pending[slot], 1u) == 1u) finish_slot(args, slot);
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
        // ---- donation: hand an untried root move to a waiting lane ----
        if (busy && E < root_e && root_e >= args.donate_min && args.donate_min > 0 &&
            ((++chk) & 15u) == 0u) {
          const int demand = static_cast<int>(ld_acquire(&args.stats->dq_head) -
                                              ld_acquire(&args.stats->dq_tail));
          if (demand > 0) {
            u64 m0, f0;
            unsigned meta0;
            fr.load(root_e, m0, f0, meta0);
            const int a0 = static_cast<signed char>((meta0 >> 6) & 0xff);
            const int b0 = static_cast<signed char>((meta0 >> 14) & 0xff);
            const int best0 = static_cast<signed char>((meta0 >> 22) & 0xff);
            const unsigned accv = ld_acquire(&args.acc[slot]);
            int lo0 = a0 > best0 ? a0 : best0;
            if (accv) {
              const int av = static_cast<int>(accv >> 8) - 128;
              if (av > lo0) lo0 = av;
            }
            const bool root_passed = (meta0 >> 30) & 1u;
            int dsq = -1;
            u64 m1 = m0;
            if (!root_passed && lo0 < b0) {
              if (meta0 >> 31) {
                const int e = list_peek(m0);
                if (e != 0xFFF) {
                  dsq = e & 63;
                  m1 = m0 + (1ULL << 60);
                }
              } else if (m0) {
                const u64 b = pick_parity(m0, ~(P0 | O0));
                dsq = ctz64(b);
                m1 = m0 ^ b;
              }
            }
            if (dsq >= 0) {
              const unsigned qi = atomicAdd(&args.stats->dq_tail, 1u);
              if (qi < args.task_cap) {
                fr.store(root_e, m1, f0, meta0);
                op = OP_DONATE;
                sq = dsq;
                dalpha = -b0;
                dbeta = -lo0;
                dq = qi;
              }
            }
          }
        }
        if (busy && op == OP_NONE) {
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

    // ---- the uniform heavy step: one flip, one mobility ----
    const bool play = op == OP_MOVE || op == OP_KEY || op == OP_DONATE;
    const bool same = op == OP_INIT || op == OP_REMASK;
    const u64 X = op == OP_DONATE ? P0 : P;
    const u64 Y = op == OP_DONATE ? O0 : O;
    const u64 bit = play ? (1ULL << sq) : 0ULL;
    const u64 f = play ? gpo_flip(X, Y, sq) : 0ULL;
    const u64 cP = same ? X : (Y ^ f);
    const u64 cO = same ? Y : (X ^ f ^ bit);
    const u64 cm = gpo_mobility(cP, cO);

    // ---- bookkeeping on the result ----
    // A node enters the keying phase (fastest-first) when it has moves and
    // at least args.ff empties: `moves` then holds the squares still to key
    // and `lst` the list being built; the list replaces `moves` when done.
    bool start_keys = false;
    if (op == OP_DONATE) {
      const unsigned qi = dq;
      const unsigned ns = n + qi;
      atomicAdd(&args.pending[slot], 1u);
      atomicExch(&args.acc[ns], 0u);
      atomicExch(&args.pending[ns], 1u);
      args.parent[qi] = slot;
      args.psq[qi] = static_cast<unsigned char>(sq);
      args.top[qi] = top;
      DonatedTask tk;
      tk.player = cP;
      tk.opp = cO;
      tk.alpha = dalpha;
      tk.beta = dbeta;
      tk.slot = ns;
      tk.pad = 0;
      args.queue[qi] = tk;
      __threadfence();
      atomicExch(&args.ready[qi], 1u);
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
        if (args.node_budget && nodes > args.node_budget) {
          // watchdog: give up on this task; its chain still completes so
          // every lane finishes, and the call reports the error
          atomicOr(&args.stats->status, kErrBudget);
          E = root_e;
          best = 0;
          alpha = beta;  // finishes at once on the next iteration
          passed = 0;
          rootbest = kMoveNoneDev;
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
}

cudaError_t batched_grid(int threads, int smem_top, int sms, int* grid, size_t* smem) {
  const int sslots = smem_top >= 2 ? smem_top - 1 : 0;
  *smem = static_cast<size_t>(threads) * sslots * kFrameBytes;
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
  const int per_block = smem_sm / per_sm - 1024;  // 1 KB per block is reserved
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
