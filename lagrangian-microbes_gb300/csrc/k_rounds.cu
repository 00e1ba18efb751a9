// K4 + K5: rock-paper-scissors species update over the step's pair set.
//
// The reference applies the pairs one after another, in place, in the iteration order of the
// Python set returned by query_pairs (interaction_simulator.py:104-105), calling
// rock_paper_scissors_interaction (interactions.py:13-40): if the two species differ, draw
// r ~ U[0,1); the cyclic winner (rock > scissors > paper > rock) wins with probability
// pRS / pSP / pPR of that matchup, and the loser takes the winner's species. Updates cascade to
// later pairs of the same step. The set order is an artifact of hashing, not a semantic.
//
// Here the order is fixed as descending pair priority (k_pairs.cu), which the CPU oracle replays
// with a restatement of the reference's pair function. Pairs that share no microbe commute, so
// any schedule that keeps the priority order at every microbe gives the same species: a pair may
// be applied as soon as it is the highest-priority unprocessed pair of both its microbes.
// r is drawn from a Philox block keyed by (ensemble seed, step, i, j) (53-bit uniform), and
// r < p is evaluated exactly as the integer test u53 < ceil(p * 2^53). The sweep that builds the
// lists makes these draws and stores the three outcomes (one per matchup) in the list entry of
// the pair's applier, so applying a pair here is a table lookup on the two species.
//
// All pairs are applied by one persistent cooperative launch without grid barriers. Each vertex v
// publishes the partner of its highest-priority unprocessed pair (NONE when it has none). A pair
// (v, u) is ready exactly when each names the other; the thread that polls the
// lower endpoint applies it and advances both. The current species, the list position and the
// partner of a vertex share one 64-bit state word, so one load tells a poller everything and the
// handoff needs no memory fence. Only the applier of a vertex's current pair ever writes that
// vertex's word, so every write has a single owner. The globally highest-priority pending pair is
// always ready, so the loop always progresses; every wait is still bounded (error flag + return
// after a timeout).
//
// When every block can own its share of the vertices in shared memory (up to 2,048 each), the
// pairs are applied by the tile-local path (rounds_tiled): handshakes between vertices of one
// block go through shared memory and only pairs crossing blocks through global memory.
//
// In pair-log runs each applied pair also gets a level = 1 + max(level of the previous pair at
// either endpoint): pairs of one level share no microbe, and (level, i, j) is a deterministic
// sequential order equal in effect to the priority order. The step's "rounds" is the max level.
#include "lm_internal.h"
#include "lm_philox.cuh"

namespace lm {

// Blocks of 1,024 threads owning two vertices each (the default) or of 512 owning four: two blocks per
// SM hold 2 x 2,048 vertices in 2 x 96 KB of shared memory. With 1,024 threads the SM keeps 2,048
// threads resident (32 registers each); the kernel is latency bound (dependent shared-memory loads,
// polls of words written by other threads), and the doubled number of resident warps shortened it
// from 74 to 66 us per launch on the first day of the 490k run and from 107 to 90 us on its last
// day. The block size is a tuning knob (lm_set_tuning); against blocks of 256 (the same vertices
// per SM) a block's range has a shorter edge for its area, so fewer pairs hand off through global
// memory.
constexpr int RD_THREADS_DEFAULT = 1024;
constexpr unsigned long long ROUNDS_TIMEOUT_NS = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Vertex state words are read and written with relaxed .gpu operations: each word is the only
// shared state a pair needs, and a word changes only through the applier of its vertex's current
// pair, so coherence of the single word is all the ordering required.
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ bool beats(int x, int y) {
  // rock(1) > scissors(3), paper(2) > rock(1), scissors(3) > paper(2)
  return (x == 1 && y == 3) || (x == 2 && y == 1) || (x == 3 && y == 2);
}

// List entry of vertex s at position h (NONE past the end); lists are read-only here.
__device__ __forceinline__ uint32_t next_partner(const Bufs& b, uint32_t s, uint32_t h) {
  const uint32_t d = b.deg[s];
  if (h >= d) return NONE;
  return d <= SLAB ? b.slab[(size_t)s * SLAB + h] : b.ovf[(size_t)b.slab[(size_t)s * SLAB] + h];
}

// The species both endpoints hold after a pair of species a and b whose applier's list entry is e
// (the reference's table, interactions.py:24-35): equal species, or a value outside {1, 2, 3},
// change nothing; otherwise the matchup's outcome bit says whether the forward winner (the species
// that beats the other) wins, and the loser takes the winner's species. The rule is symmetric in
// the two endpoints, so the bit needs no orientation.
__device__ __forceinline__ int rps_outcome(int a, int b, uint32_t e) {
  if (a == b || a < 1 || a > 3 || b < 1 || b > 3) return -1;  // no change
  const int c = (a + b == 4) ? 0 : (a + b == 3) ? 1 : 2;  // {1,3} rock/scissors, {1,2} paper/rock, {2,3}
  const bool fwd_wins = (e >> (ENTRY_WIN_SHIFT + c)) & 1u;
  return beats(a, b) == fwd_wins ? a : b;
}

// Apply pair (s, u), s < u in cell order, whose state words ws, wu name each other. Everything
// the pair needs that other threads write (both species, both list positions) is inside the two
// words, so no fence is needed: the next applier of either vertex reads the words this one
// stores. Returns the pair's level when levels are tracked (pair-log runs), else 0.
__device__ __forceinline__ uint32_t apply_pair(const Bufs& b, uint32_t s, uint32_t u, unsigned long long ws,
                                               unsigned long long wu, Ctrl* ctrl) {
  const uint32_t hs = state_pos(ws), hu = state_pos(wu);
  const uint32_t ns = next_partner(b, s, hs + 1u), nu = next_partner(b, u, hu + 1u);
  const uint32_t pa = b.sid[s], pb = b.sid[u];
  const int o = rps_outcome(state_species(ws), state_species(wu), state_partner(ws));
  const int new_s = o < 0 ? state_species(ws) : o, new_u = o < 0 ? state_species(wu) : o;
  const uint32_t pi = min(pa, pb), pj = max(pa, pb);
  uint32_t level = 0;
  if (b.plog) {  // pair-log runs: levels live outside the state words, so order them with fences
    __threadfence();
    level = max(__ldcg(b.level + s), __ldcg(b.level + u)) + 1u;
    __stcg(b.level + s, level);
    __stcg(b.level + u, level);
    const uint32_t k = atomicAdd(&ctrl->plog_n, 1u);
    if (k < b.plog_cap) {
      b.plog[3 * k + 0] = pi;
      b.plog[3 * k + 1] = pj;
      b.plog[3 * k + 2] = level - 1u;
    }
    __threadfence();
  }
  // a vertex whose list is done keeps its final species in the species array
  if (nu == NONE) b.species[pb] = (int8_t)new_u;
  if (ns == NONE) b.species[pa] = (int8_t)new_s;
  st_relaxed(b.wstate + u, pack_state(nu, hu + 1u, new_u));
  st_relaxed(b.wstate + s, pack_state(ns, hs + 1u, new_s));
  return level;
}

constexpr int POLL_BATCH = 2;  // vertices whose state words one thread loads before testing them

// ---- tile-local interaction: block-owned vertex ranges with handshakes in shared memory ----
//
// Cell keys are tile-major, so a contiguous range of cell-ordered vertices is a compact 2D patch.
// Block b owns the vertices [b V, b V + V) (V <= TL_VMAX: an equal share in whole warps) and keeps their state words,
// slot ids, degrees and list entries in shared memory. A pair whose two microbes the block owns
// hands off through shared memory (tens of cycles instead of an L2 round trip); a pair that
// crosses blocks goes through the global state words: the vertex's word is published there while
// its current partner is outside the block, the owner of the lower endpoint applies the pair and
// writes the other endpoint's global word, and that endpoint's owner pulls the change back into
// shared memory. As in the global path, only the applier of a vertex's current pair writes the
// vertex's word, so no fences are needed.
static_assert(SLAB == 8, "the tile path copies a slab row as two 16-byte loads");
constexpr uint32_t TL_VMAX = 2048;                     // vertices per block at most
constexpr size_t TL_SMEM = TL_VMAX * (8 + 4 + 4 + 4 * SLAB);  // words, slot ids, degrees, lists

__device__ __forceinline__ unsigned long long ld_sh(const unsigned long long* p) {
  return *(const volatile unsigned long long*)p;
}
__device__ __forceinline__ void st_sh(unsigned long long* p, unsigned long long v) {
  *(volatile unsigned long long*)p = v;
}

struct TileSmem {
  unsigned long long* w;  // [TL_VMAX] state words
  uint32_t* sid;          // [TL_VMAX] slot ids
  uint32_t* deg;          // [TL_VMAX] list lengths
  uint32_t* lst;          // [SLAB][TL_VMAX] list entries (slab vertices) / [0][l] = overflow offset
};

// Entry h of the list of local vertex l (NONE past the end).
__device__ __forceinline__ uint32_t tl_entry(const Bufs& b, const TileSmem& t, uint32_t l, uint32_t h) {
  const uint32_t d = t.deg[l];
  if (h >= d) return NONE;
  return d <= SLAB ? t.lst[h * TL_VMAX + l] : b.ovf[(size_t)t.lst[l] + h];
}

// The pairs among cell-order vertices [g_lo, g_hi) (a group of whole ensembles, so no pair leaves
// it), at most TL_VMAX per block: each block owns an equal share, in whole warps. Every block of the
// grid takes part (whole 1,024-vertex columns left 64 of the 304 blocks idle at 490k, and all but a
// few idle for a small ensemble run alone).
template <int RD_THREADS>
__device__ void tl_group(const Bufs& b, uint32_t step, Ctrl* ctrl, unsigned long long t0, uint32_t g_lo,
                         uint32_t g_hi) {
  constexpr int TL_VPT = (int)TL_VMAX / RD_THREADS;  // vertices per thread at most
  extern __shared__ unsigned long long tl_raw[];
  TileSmem t;
  t.w = tl_raw;
  t.sid = reinterpret_cast<uint32_t*>(t.w + TL_VMAX);
  t.deg = t.sid + TL_VMAX;
  t.lst = t.deg + TL_VMAX;
  const uint32_t n_g = g_hi - g_lo;
  // every block gets an equal share, rounded up to whole warps (at most TL_VMAX: the caller checked
  // that the group fits the grid's shared memory)
  const uint32_t V = min(TL_VMAX, max(32u, (((n_g + gridDim.x - 1) / gridDim.x) + 31u) & ~31u));
  const uint32_t lo = min(g_hi, g_lo + blockIdx.x * V);
  const uint32_t hi = min(g_hi, lo + V);
  const uint32_t nloc = hi - lo;
  // every load of the set-up is independent: the whole slab row (two 16-byte loads; entries past
  // the degree are never read; slot 0 of a long list is its overflow offset), for all of the
  // thread's vertices at once
#pragma unroll
  for (int k = 0; k < TL_VPT; ++k) {
    const uint32_t l = threadIdx.x + (uint32_t)k * RD_THREADS;
    if (l < nloc) {
      const uint32_t s = lo + l;
      const unsigned long long w0 = ld_relaxed(b.wstate + s);  // written by the sweep, which published every first pair
      const uint32_t sid = b.sid[s], d = b.deg[s];
      const uint4* row = reinterpret_cast<const uint4*>(b.slab + (size_t)s * SLAB);
      const uint4 r0 = row[0], r1 = row[1];
      t.w[l] = w0;
      t.sid[l] = sid;
      t.deg[l] = d;
      t.lst[0 * TL_VMAX + l] = r0.x, t.lst[1 * TL_VMAX + l] = r0.y, t.lst[2 * TL_VMAX + l] = r0.z;
      t.lst[3 * TL_VMAX + l] = r0.w, t.lst[4 * TL_VMAX + l] = r1.x, t.lst[5 * TL_VMAX + l] = r1.y;
      t.lst[6 * TL_VMAX + l] = r1.z, t.lst[7 * TL_VMAX + l] = r1.w;
    }
  }
  __syncthreads();
  uint32_t live = 0;
  for (int k = 0; k < TL_VPT; ++k)
    if (threadIdx.x + (uint32_t)k * RD_THREADS < nloc) live |= 1u << k;
  uint32_t polls = 0;
  while (live) {
#pragma unroll
    for (int k = 0; k < TL_VPT; ++k) {
      if (!((live >> k) & 1u)) continue;
      const uint32_t l = threadIdx.x + (uint32_t)k * RD_THREADS, s = lo + l;
      const unsigned long long ws = ld_sh(t.w + l);
      const uint32_t ue = state_partner(ws);  // s's current list entry
      if (ue == NONE) {
        live &= ~(1u << k);
        continue;
      }
      const uint32_t u = entry_id(ue);
      const bool u_local = u >= lo && u < hi;
      if (s > u) {
        // the owner of u applies; while u is outside the block, take the result from global memory.
        // Positions only grow: a global word behind the shared one (published a moment after a
        // local apply wrote the shared word, or left from an earlier publish) is not taken.
        if (!u_local) {
          const unsigned long long g = ld_relaxed(b.wstate + s);
          if (state_pos(g) > state_pos(ws)) st_sh(t.w + l, g);
        }
        continue;
      }
      const unsigned long long wu = u_local ? ld_sh(t.w + (u - lo)) : ld_relaxed(b.wstate + u);
      if (state_partner(wu) != s) continue;  // u's entry of a pair it does not apply carries no bits
      // apply (s, u): this thread owns the lower endpoint
      const uint32_t hs = state_pos(ws), hu = state_pos(wu);
      const uint32_t ns = tl_entry(b, t, l, hs + 1u);
      uint32_t nu;
      if (u_local) {
        nu = tl_entry(b, t, u - lo, hu + 1u);
      } else {
        const uint32_t du = b.deg[u];
        nu = hu + 1u < du ? (du <= SLAB ? b.slab[(size_t)u * SLAB + hu + 1u] : b.ovf[(size_t)b.slab[(size_t)u * SLAB] + hu + 1u]) : NONE;
      }
      const int o = rps_outcome(state_species(ws), state_species(wu), ue);
      const int new_s = o < 0 ? state_species(ws) : o, new_u = o < 0 ? state_species(wu) : o;
      const unsigned long long nwu = pack_state(nu, hu + 1u, new_u), nws = pack_state(ns, hs + 1u, new_s);
      const uint32_t nu_id = entry_id(nu), ns_id = entry_id(ns);
      if (u_local) {
        st_sh(t.w + (u - lo), nwu);
        if (nu != NONE && (nu_id < lo || nu_id >= hi)) st_relaxed(b.wstate + u, nwu);  // u's next pair crosses
      } else {
        st_relaxed(b.wstate + u, nwu);  // u's owner pulls it
      }
      st_sh(t.w + l, nws);
      if (ns != NONE && (ns_id < lo || ns_id >= hi)) st_relaxed(b.wstate + s, nws);  // s's next pair crosses
    }
    if (live && ((++polls & 63u) == 0u) && globaltimer() - t0 > ROUNDS_TIMEOUT_NS) {
      atomicOr(&ctrl->err, (uint32_t)ERRB_TIMEOUT);
      break;
    }
  }
  // every owned list is done (its word names no partner, and no one writes a vertex's word after
  // its last pair): the words hold the final species, written back once per vertex
#pragma unroll
  for (int k = 0; k < TL_VPT; ++k) {
    const uint32_t l = threadIdx.x + (uint32_t)k * RD_THREADS;
    if (l < nloc && t.deg[l]) b.species[t.sid[l]] = (int8_t)state_species(ld_sh(t.w + l));
  }
}

// Groups of whole ensembles (consecutive in cell order) whose vertices fit the blocks' shared
// memory, run one after another by every block. No barrier separates the groups: pairs never join
// two ensembles, and a block that is still in group g while another has moved to g + 1 only
// delays the handoffs of g + 1 that cross into it, whose words it loads from global memory when it
// gets there (the same rule that covers blocks starting at different times).
constexpr int TL_GROUPS_MAX = 64;

// Returns false (nothing done) when the step does not fit the tile path (grid-uniform).
template <int RD_THREADS>
__device__ bool rounds_tiled(const Bufs& b, uint32_t step, Ctrl* ctrl, unsigned long long t0, uint32_t n_valid) {
  if (b.plog) return false;
  const uint32_t cap = gridDim.x * TL_VMAX;
  __shared__ uint32_t gb[TL_GROUPS_MAX + 1];
  __shared__ int ng;
  if (n_valid <= cap) {
    if (threadIdx.x == 0) {
      gb[0] = 0;
      gb[1] = n_valid;
      ng = 1;
    }
  } else {
    // the k-th ensemble in key order, e = eord[k], holds the vertices from cstart[cell_base_e] to
    // the next one's start; greedy groups of whole ensembles consecutive in that order, each at
    // most `cap` vertices (none when one ensemble alone is larger)
    extern __shared__ unsigned long long tl_raw[];
    uint32_t* es = reinterpret_cast<uint32_t*>(tl_raw);
    const uint32_t E = b.n_ens;
    const bool fits = E + 1 <= (uint32_t)(TL_SMEM / sizeof(uint32_t));
    if (fits) {
      for (uint32_t e = threadIdx.x; e < E; e += blockDim.x) es[e] = b.cstart[b.grids[b.eord[e]].cell_base];
      if (threadIdx.x == 0) es[E] = n_valid;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      bool ok = fits;
      int g = 0;  // the open group starts at gb[g]
      if (ok) gb[0] = es[0];
      for (uint32_t e = 1; e <= E && ok; ++e) {
        if (es[e] - gb[g] <= cap) continue;  // ensemble e - 1 fits the open group
        if (es[e - 1] != gb[g]) {            // close the group before ensemble e - 1
          if (g + 1 >= TL_GROUPS_MAX) {
            ok = false;
            break;
          }
          gb[++g] = es[e - 1];
        }
        ok = es[e] - gb[g] <= cap;  // else ensemble e - 1 alone is larger than the blocks hold
      }
      if (ok) gb[g + 1] = n_valid;
      ng = ok ? g + 1 : 0;  // groups [gb[k], gb[k + 1]), k < ng
    }
  }
  __syncthreads();
  const int groups = ng;
  if (groups <= 0) return false;
  for (int g = 0; g < groups; ++g) {
    tl_group<RD_THREADS>(b, step, ctrl, t0, gb[g], gb[g + 1]);
    __syncthreads();  // the block's shared lists are reused by the next group
  }
  return true;
}

template <int RD_THREADS>
__global__ void __launch_bounds__(RD_THREADS, 2) k_rounds(Bufs b, StepArgs a, Ctrl* ctrl) {
  pdl_wait();
  // the control words, read by one thread per block: every thread of the 300-odd blocks loading
  // the same L2 line (the loads are volatile, so L1 does not merge them) queued ~10^4 requests on
  // one L2 slice and delayed the start of the pairs by 4-10 us
  __shared__ uint32_t cw[4];
  if (threadIdx.x == 0) {
    cw[0] = ((volatile uint32_t*)&ctrl->halt)[0];
    cw[1] = ((volatile uint32_t*)&ctrl->act_n)[0];
    cw[2] = ((volatile uint32_t*)&ctrl->n_valid)[0];
    cw[3] = a.use_ctrl_step ? ((volatile uint32_t*)&ctrl->step)[0] : a.step0;
  }
  __syncthreads();
  if (cw[0]) return;
  if (a.test_wait_ns) {
    // injected failure (tests): the wait of a stalled dependency, on a flag that nothing sets,
    // bounded like every wait of this kernel; the step applies no pair and reports the timeout
    if (threadIdx.x == 0) {
      const unsigned long long w0 = globaltimer();
      while (((volatile uint32_t*)&ctrl->never)[0] == 0u) {
        if (globaltimer() - w0 > a.test_wait_ns) {
          atomicOr(&ctrl->err, (uint32_t)ERRB_TIMEOUT);
          break;
        }
      }
    }
    return;
  }
  const uint32_t step = cw[3];
  const uint32_t cnt = cw[1];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t max_level = 0;
  const unsigned long long t0 = globaltimer();
  if (rounds_tiled<RD_THREADS>(b, step, ctrl, t0, cw[2])) return;  // levels are tracked only in pair-log runs
  uint32_t polls = 0;
  if (cnt <= (uint32_t)POLL_BATCH * stride) {
    // every thread owns at most POLL_BATCH vertices: keep their ids in registers and stop polling
    // a vertex once its list is done (its partner stays NONE from then on)
    uint32_t sv[POLL_BATCH];
    uint32_t live = 0;
#pragma unroll
    for (int k = 0; k < POLL_BATCH; ++k) {
      const uint32_t x = first + (uint32_t)k * stride;
      sv[k] = x < cnt ? b.act[x] : NONE;
      if (sv[k] != NONE) live |= 1u << k;
    }
    while (live) {
      unsigned long long ws[POLL_BATCH], wu[POLL_BATCH];
#pragma unroll
      for (int k = 0; k < POLL_BATCH; ++k)
        ws[k] = (live >> k) & 1u ? ld_relaxed(b.wstate + sv[k]) : (unsigned long long)NONE;
#pragma unroll
      for (int k = 0; k < POLL_BATCH; ++k) {
        const uint32_t u = entry_id(state_partner(ws[k]));
        wu[k] = NONE;
        if (state_partner(ws[k]) == NONE) live &= ~(1u << k);
        else if (sv[k] < u) wu[k] = ld_relaxed(b.wstate + u);
      }
#pragma unroll
      for (int k = 0; k < POLL_BATCH; ++k) {
        const uint32_t u = entry_id(state_partner(ws[k]));
        if (state_partner(ws[k]) != NONE && sv[k] < u && state_partner(wu[k]) == sv[k])
          max_level = max(max_level, apply_pair(b, sv[k], u, ws[k], wu[k], ctrl));
      }
      if (live && ((++polls & 63u) == 0u) && globaltimer() - t0 > ROUNDS_TIMEOUT_NS) {
        atomicOr(&ctrl->err, (uint32_t)ERRB_TIMEOUT);
        break;
      }
    }
  }
  bool pending = first < cnt && cnt > (uint32_t)POLL_BATCH * stride;
  while (pending) {
    pending = false;
    for (uint32_t x0 = first; x0 < cnt; x0 += POLL_BATCH * stride) {
      uint32_t sv[POLL_BATCH];
      unsigned long long ws[POLL_BATCH], wu[POLL_BATCH];
#pragma unroll
      for (int k = 0; k < POLL_BATCH; ++k) {
        const uint32_t x = x0 + (uint32_t)k * stride;
        sv[k] = x < cnt ? b.act[x] : NONE;
        ws[k] = sv[k] != NONE ? ld_relaxed(b.wstate + sv[k]) : (unsigned long long)NONE;
      }
#pragma unroll
      for (int k = 0; k < POLL_BATCH; ++k) {
        const uint32_t u = entry_id(state_partner(ws[k]));
        wu[k] = NONE;
        if (state_partner(ws[k]) != NONE) {
          pending = true;
          if (sv[k] < u) wu[k] = ld_relaxed(b.wstate + u);
        }
      }
#pragma unroll
      for (int k = 0; k < POLL_BATCH; ++k) {
        const uint32_t u = entry_id(state_partner(ws[k]));
        if (state_partner(ws[k]) != NONE && sv[k] < u && state_partner(wu[k]) == sv[k])
          max_level = max(max_level, apply_pair(b, sv[k], u, ws[k], wu[k], ctrl));
      }
    }
    if (pending && ((++polls & 63u) == 0u) && globaltimer() - t0 > ROUNDS_TIMEOUT_NS) {
      atomicOr(&ctrl->err, (uint32_t)ERRB_TIMEOUT);
      break;
    }
  }
  for (int o = 16; o > 0; o >>= 1) max_level = max(max_level, __shfl_xor_sync(0xffffffffu, max_level, o));
  if ((threadIdx.x & 31) == 0 && max_level) {
    atomicMax(&ctrl->rounds, max_level);
    atomicMax(&ctrl->max_rounds, max_level);
  }
}

// Blocks per SM of the interaction kernel with `threads` per block (512 or 1,024).
template <int T>
static int rounds_per_sm(int device) {
  int per_sm = 0;
  cudaFuncSetAttribute(k_rounds<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TL_SMEM);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rounds<T>, T, TL_SMEM);
  (void)device;
  return per_sm;
}

int rounds_grid(int device, int threads, int* block) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (threads != 512) threads = RD_THREADS_DEFAULT;
  int per_sm = threads == 512 ? rounds_per_sm<512>(device) : rounds_per_sm<1024>(device);
  if (per_sm < 1) per_sm = 1;
  if (per_sm > 4) per_sm = 4;
  *block = threads;
  return sms * per_sm;
}

cudaError_t launch_rounds(const Bufs& b, const StepArgs& a, Ctrl* ctrl, int grid, int block, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = TL_SMEM;  // the tile-local path's vertex state
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (block == 512) return cudaLaunchKernelEx(&cfg, k_rounds<512>, b, a, ctrl);
  return cudaLaunchKernelEx(&cfg, k_rounds<1024>, b, a, ctrl);
}

// Species counts after the step, per ensemble and in total ([0] collects values outside 1..3).
__global__ void __launch_bounds__(SLOT_BLOCK) k_census(Bufs b, Ctrl* ctrl) {
  pdl_wait();
  if (ctrl->halt) return;
  __shared__ uint32_t h[4];
  if (threadIdx.x < 4) h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t p = blockIdx.x * SLOT_BLOCK + threadIdx.x;
  int s = -1;
  if (p < b.nslots && b.status[p] != STATUS_PAD) {
    s = b.species[p];
    s = (s >= 1 && s <= 3) ? s : 0;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    uint32_t v = __popc(__ballot_sync(0xffffffffu, s == k));
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&h[k], v);
  }
  __syncthreads();
  if (threadIdx.x < 4 && h[threadIdx.x]) {
    atomicAdd(&b.census[4 * b.block_ens[blockIdx.x] + threadIdx.x], h[threadIdx.x]);
    atomicAdd(&ctrl->census[threadIdx.x], h[threadIdx.x]);
  }
}

const void* lm_census_kernel() { return (const void*)k_census; }

void launch_census(const Bufs& b, Ctrl* ctrl, cudaStream_t st) {
  if (b.nslots == 0) return;
  launch_dep(k_census, dim3((b.nslots + SLOT_BLOCK - 1) / SLOT_BLOCK), dim3(SLOT_BLOCK), st, b, ctrl);
}

}  // namespace lm
