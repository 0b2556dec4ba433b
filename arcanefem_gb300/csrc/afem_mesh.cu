// Connectivity and sparsity for P1 meshes.
//
// node -> cell adjacency (the transpose of cell -> node):
//   histogram of incidences, exclusive scan, scatter, then a per-node
//   segmented sort of (cell, local) keys so that cells come out ascending --
//   the order of Arcane's nodeCell() connectivity.  The histogram uses
//   integer atomics on per-node counters and each incidence keeps its atomic's
//   result as its place in the node's list (no atomic in the scatter); the
//   segmented sort (a bitonic network, in one thread's registers or across
//   a warp's lanes) makes the result independent of the atomics' order, so
//   the output is deterministic.
//
// node -> node sparsity (rows of the assembled matrix):
//   8 lanes per node (4 nodes per warp) on meshes of many cells per node,
//   one thread per node on meshes of few, one warp per node for the rows
//   either passes on: the nodes of the node's incident cells go into a hash
//   set in shared memory; the number of
//   distinct values is the row length = 1 + number of neighbours
//   (femutils/BSRFormat.cc:445-557, row = deg + 1).  The same pass ranks
//   each neighbour, writes the columns (ascending or self-last) and, for
//   every cell-node incidence, its position in the row (the slot map used by
//   the assembly kernels) in one packed store.  afem_sparsity_rows runs it
//   before the row starts are known, with each row at a padded offset
//   ((npc - 1) * nc_ptr[n] + n bounds the rows before n), into a buffer the
//   context keeps; afem_sparsity_cols then copies the rows into place, or,
//   for other mesh arrays, runs the pass again with the real row starts.
//   Rows may hold up to 255 entries (the slot map is uint8); longer rows are
//   reported as mesh errors.
#include <algorithm>
#include <climits>
#include <type_traits>

#include "afem_internal.cuh"

namespace afem {

// ---------------------------------------------------------------------------
// node -> cell

// Histogram of incidences per node; each incidence keeps the count its
// atomic returned (its rank among the node's incidences, in arbitrary order),
// so that the scatter needs no second atomic.
__global__ void k_nc_count(const int32_t* __restrict__ cn, int64_t total, int nb_node, int32_t* __restrict__ cnt,
                           int32_t* __restrict__ rank, int* __restrict__ err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t n = cn[i];
    if (n < 0 || n >= nb_node) {
      atomicOr(err, 1);
      continue;
    }
    rank[i] = atomicAdd(&cnt[n], 1);
  }
}

__global__ void k_nc_scatter(const int32_t* __restrict__ cn, int64_t total, int npc, int nb_node,
                             const int32_t* __restrict__ nc_ptr, const int32_t* __restrict__ rank,
                             int32_t* __restrict__ key) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t n = cn[i];
    if (n < 0 || n >= nb_node) continue;
    int32_t pos = nc_ptr[n] + rank[i];
    int32_t cell = (int32_t)(i / npc);
    int32_t local = (int32_t)(i - (int64_t)cell * npc);
    key[pos] = (cell << 3) | local;  // cells < 2^28 checked by the caller; local < 8
  }
}

// Ascending sort of M keys in registers (bitonic network, M a power of two).
template <int M>
__device__ __forceinline__ void bitonic_sort(uint32_t (&a)[M]) {
#pragma unroll
  for (int k = 2; k <= M; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
      for (int i = 0; i < M; ++i) {
        const int l = i ^ j;
        if (l > i) {
          const uint32_t lo = min(a[i], a[l]), hi = max(a[i], a[l]);
          a[i] = (i & k) == 0 ? lo : hi;
          a[l] = (i & k) == 0 ? hi : lo;
        }
      }
    }
  }
}

// Per-node sort of the (cell << 3 | local) keys, then split; the inverse map
// records, for each (cell, local), its incidence index.  One thread per node
// (meshes of at most 16 cells per node on average: triangles, hexahedra):
// up to 32 keys are sorted by a bitonic network in registers; longer lists
// (rare hubs) by an insertion sort in place.
__global__ void k_nc_sort_thread(int nb_node, int npc, const int32_t* __restrict__ nc_ptr, int32_t* __restrict__ key,
                          int32_t* __restrict__ nc_cell, uint8_t* __restrict__ nc_local,
                          int32_t* __restrict__ nc_inverse) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nb_node; n += gridDim.x * blockDim.x) {
    const int32_t b = nc_ptr[n], e = nc_ptr[n + 1];
    const int deg = e - b;
    if (deg <= 32) {
      uint32_t a[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) a[i] = i < deg ? (uint32_t)key[b + i] : 0xffffffffu;
      bitonic_sort<32>(a);
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        if (i < deg) {
          const int32_t v = (int32_t)a[i];
          nc_cell[b + i] = v >> 3;
          nc_local[b + i] = (uint8_t)(v & 7);
          if (nc_inverse) nc_inverse[(int64_t)(v >> 3) * npc + (v & 7)] = b + i;
        }
      }
    } else {
      for (int32_t i = b + 1; i < e; ++i) {
        const int32_t v = key[i];
        int32_t j = i - 1;
        while (j >= b && key[j] > v) {
          key[j + 1] = key[j];
          --j;
        }
        key[j + 1] = v;
      }
      for (int32_t i = b; i < e; ++i) {
        const int32_t v = key[i];
        nc_cell[i] = v >> 3;
        nc_local[i] = (uint8_t)(v & 7);
        if (nc_inverse) nc_inverse[(int64_t)(v >> 3) * npc + (v & 7)] = i;
      }
    }
  }
}

constexpr int kWarpsPerBlock = 8;

// The same with one warp per node (meshes of more than 16 cells per node on
// average: its loads and stores stay coalesced over the node's list):
// up to 32 keys are sorted by a bitonic network on registers (shuffles);
// longer lists (rare) by an insertion sort in lane 0.
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_nc_sort_warp(int nb_node, int npc,
                                                                 const int32_t* __restrict__ nc_ptr,
                                                                 int32_t* __restrict__ key,
                                                                 int32_t* __restrict__ nc_cell,
                                                                 uint8_t* __restrict__ nc_local,
                                                                 int32_t* __restrict__ nc_inverse) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int n = wid; n < nb_node; n += nwarps) {
    const int32_t b = nc_ptr[n], e = nc_ptr[n + 1];
    const int deg = e - b;
    if (deg <= 32) {
      int32_t v = lane < deg ? key[b + lane] : INT_MAX;
#pragma unroll
      for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
          int32_t o = __shfl_xor_sync(0xffffffffu, v, j);
          bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
          v = keep_min ? min(v, o) : max(v, o);
        }
      }
      if (lane < deg) key[b + lane] = v;
    } else if (lane == 0) {
      for (int32_t i = b + 1; i < e; ++i) {
        int32_t v = key[i];
        int32_t j = i - 1;
        while (j >= b && key[j] > v) {
          key[j + 1] = key[j];
          --j;
        }
        key[j + 1] = v;
      }
    }
    __syncwarp();
    for (int32_t i = b + lane; i < e; i += 32) {
      int32_t v = key[i];
      nc_cell[i] = v >> 3;
      nc_local[i] = (uint8_t)(v & 7);
      if (nc_inverse) nc_inverse[(int64_t)(v >> 3) * npc + (v & 7)] = i;
    }
  }
}

// ---------------------------------------------------------------------------
// node -> node

constexpr int kMaxRowLen = 255;   // slot map entries are uint8
constexpr int kTabSlots = 256;    // hash table entries per warp: every distinct neighbour of a row fits

__device__ __forceinline__ int tab_hash(int32_t v) { return (int)(((uint32_t)v * 2654435761u) >> 24); }

// Per-warp tables in shared memory.  key: open-addressing hash set of the
// row's neighbours (-1 = empty; linear probing); at: the table slot of each
// distinct neighbour in order of first insertion (for the ranks and to clear
// the table afterwards); val: the neighbours in that order, padded with
// INT_MAX for the 4-wide rank loop; pos: the position in the row of the
// neighbour held in each table slot.
struct RowTables {
  int32_t* key;
  int16_t* at;
  int32_t* val;
  uint8_t* pos;
};

// Inserts v; returns its table slot (fresh: first insertion), or -1 when
// the table is full.
__device__ __forceinline__ int tab_insert(int32_t* key, int32_t v, bool& fresh) {
  int h = tab_hash(v);
  for (int p = 0; p < kTabSlots; ++p, h = (h + 1) & (kTabSlots - 1)) {
    const int32_t old = atomicCAS(key + h, -1, v);
    if (old == -1) {
      fresh = true;
      return h;
    }
    if (old == v) return h;
  }
  return -1;
}

// v[j] for a run-time j in [0, NPC), by selects (no local-memory array)
template <int NPC>
__device__ __forceinline__ int32_t pick(const int32_t (&v)[NPC], int j) {
  int32_t x = v[0];
#pragma unroll
  for (int q = 1; q < NPC; ++q)
    if (j == q) x = v[q];
  return x;
}

__device__ __forceinline__ int tab_find(const int32_t* key, int32_t v) {
  int h = tab_hash(v);
  for (int p = 0; p < kTabSlots; ++p, h = (h + 1) & (kTabSlots - 1))
    if (key[h] == v) return h;
  return 0;   // not reached: every neighbour was inserted
}

// One thread per node.  Its hash set of neighbours lives in shared memory,
// interleaved across the block's threads (slot h of thread t at key[h][t]),
// so that the 32 probes of a warp fall in 32 distinct banks whatever their
// slots.  The thread streams its node's incidences in increasing order, the
// cell nodes of each loaded two incidences ahead (CellStream), and inserts
// the nodes other than n of each cell: the number of first insertions D is
// the number of distinct neighbours and the row holds D + 1 entries (the
// node itself included, as the reference's deg + 1 rows,
// femutils/BSRFormat.cc:445-557).  With FILL the row is then written: the
// neighbours, tagged with their insertion index, are sorted by a bitonic
// network in registers (rows of up to 16 neighbours, 32 for hexahedra;
// longer ones rank each neighbour by counting the smaller ones), which gives
// each column's position in either order, and every incidence writes its
// NPC slot bytes (its own column first, then the other cell nodes in
// increasing local index) in one packed store.  A row with more neighbours
// than the table's 3/4 is appended to `defer` for k_sparsity_rows_warp, and
// so are the light nodes of a warp that holds too few of them.
// Errors: bit 2 a row of more than kMaxRowLen entries, bit 4 a row_ptr that
// does not match, bit 8 a node id out of range.
constexpr int kThreadBlock = 128;
// A warp of k_sparsity_thread with fewer light nodes than this passes them on.
constexpr int kThreadMinLanes = 12;

template <int NPC>
struct ThreadTable {
  static constexpr int slots = NPC == 8 ? 64 : 32;   // power of two
  static constexpr int max_d = slots * 3 / 4;        // load factor at most 3/4
  // Nodes in more cells than this go to k_sparsity_rows_warp, whose lanes
  // then stay at least half busy and read the cells of one node together
  // (tetrahedral meshes: about 24 cells per node, the others 4 to 8).
  static constexpr int max_deg = 16;
  // rows of at most sort_m neighbours are ranked by the sorting network, the
  // insertion index in the low sort_bits bits of each key
  static constexpr int sort_m = NPC == 8 ? 32 : 16;
  static constexpr int sort_bits = NPC == 8 ? 5 : 4;
};

__device__ __forceinline__ void defer_node(int n, int32_t* defer, int32_t* defer_count) {
  defer[atomicAdd(defer_count, 1)] = n;
}

// The nodes of cell c (one or two 16-byte loads when cn is 16-byte aligned).
template <int NPC>
__device__ __forceinline__ void load_cell(const int32_t* __restrict__ cn, bool vec, int32_t c, int32_t (&v)[NPC]) {
  const int32_t* cp = cn + (int64_t)c * NPC;
  if constexpr (NPC == 4 || NPC == 8) {
    if (vec) {
#pragma unroll
      for (int k = 0; k < NPC / 4; ++k) {
        const int4 q = __ldg(reinterpret_cast<const int4*>(cp) + k);
        v[4 * k] = q.x;
        v[4 * k + 1] = q.y;
        v[4 * k + 2] = q.z;
        v[4 * k + 3] = q.w;
      }
      return;
    }
  }
#pragma unroll
  for (int j = 0; j < NPC; ++j) v[j] = __ldg(cp + j);
}

// The cells of incidences b, b + 1, ... < e in order: the nodes (and the
// local index of the row's node) two incidences ahead, the cell ids three
// ahead, so that a thread's dependent loads overlap its work on the earlier
// incidences.
template <int NPC>
struct CellStream {
  int32_t v0[NPC], v1[NPC];
  int32_t c2, l0, l1;
  __device__ __forceinline__ void start(const int32_t* __restrict__ cn, const int32_t* __restrict__ nc_cell,
                                        const uint8_t* __restrict__ nc_local, bool vec, int32_t b, int32_t e) {
#pragma unroll
    for (int j = 0; j < NPC; ++j) v0[j] = v1[j] = 0;
    l0 = l1 = 0;
    const int32_t c0 = b < e ? __ldg(nc_cell + b) : 0;
    const int32_t c1 = b + 1 < e ? __ldg(nc_cell + b + 1) : 0;
    c2 = b + 2 < e ? __ldg(nc_cell + b + 2) : 0;
    if (b < e) load_cell<NPC>(cn, vec, c0, v0);
    if (b + 1 < e) load_cell<NPC>(cn, vec, c1, v1);
    if (nc_local) {
      if (b < e) l0 = __ldg(nc_local + b);
      if (b + 1 < e) l1 = __ldg(nc_local + b + 1);
    }
  }
  // incidence p (b <= p < e): its cell nodes into v and its local index
  __device__ __forceinline__ int next(const int32_t* __restrict__ cn, const int32_t* __restrict__ nc_cell,
                                      const uint8_t* __restrict__ nc_local, bool vec, int32_t p, int32_t e,
                                      int32_t (&v)[NPC]) {
    const int li = l0;
#pragma unroll
    for (int j = 0; j < NPC; ++j) {
      v[j] = v0[j];
      v0[j] = v1[j];
    }
    l0 = l1;
    if (p + 2 < e) {
      load_cell<NPC>(cn, vec, c2, v1);
      if (nc_local) l1 = __ldg(nc_local + p + 2);
    }
    if (p + 3 < e) c2 = __ldg(nc_cell + p + 3);
    return li;
  }
};


// Local index of node n in a cell (its first occurrence).  Without the
// node -> cell local indices (afem_sparsity_rows) the slot bytes take n's
// place from the cell itself; a cell that holds n twice is flagged (bit 16),
// since there the two ways of numbering differ.
template <int NPC>
__device__ __forceinline__ int local_index(const int32_t (&v)[NPC], int32_t n, int* err) {
  int li = -1, hits = 0;
#pragma unroll
  for (int j = NPC - 1; j >= 0; --j)
    if (v[j] == n) {
      li = j;
      ++hits;
    }
  if (hits != 1) atomicOr(err, 16);
  return li < 0 ? 0 : li;
}

template <int NPC, bool FILL>
__global__ void __launch_bounds__(kThreadBlock)
    k_sparsity_thread(int nb_node, const int32_t* __restrict__ cn, const int32_t* __restrict__ nc_ptr,
                      const int32_t* __restrict__ nc_cell, const uint8_t* __restrict__ nc_local,
                      const int32_t* __restrict__ row_ptr, int self_last, int packed_slots,
                      int32_t* __restrict__ row_len, int32_t* __restrict__ cols, uint8_t* __restrict__ slot,
                      int32_t* __restrict__ defer, int32_t* __restrict__ defer_count, int* __restrict__ err) {
  using TT = ThreadTable<NPC>;
  constexpr int TS = TT::slots, DMAX = TT::max_d, M = TT::sort_m, SB = TT::sort_bits;
  __shared__ int32_t s_key[TS][kThreadBlock];
  __shared__ uint8_t s_at[DMAX][kThreadBlock];              // table slot of each neighbour, in order of insertion
  __shared__ uint8_t s_pos[FILL ? TS : 1][kThreadBlock];     // position in the row, by table slot
  const int t = threadIdx.x;
#pragma unroll
  for (int h = 0; h < TS; ++h) s_key[h][t] = -1;
  const int lane = t & 31;
  const bool vec = (reinterpret_cast<uintptr_t>(cn) & 15) == 0;
  // node ids below 2^(31 - SB) leave room for the insertion index in a sort key
  const bool small_ids = nb_node <= (1 << (31 - SB));
  for (int n0 = blockIdx.x * kThreadBlock + (t & ~31); n0 < nb_node; n0 += gridDim.x * kThreadBlock) {
    const int n = n0 + lane;
    int32_t b = 0, e = 0;
    if (n < nb_node) {
      b = __ldg(nc_ptr + n);
      e = __ldg(nc_ptr + n + 1);
    }
    const bool light = n < nb_node && e - b <= TT::max_deg;   // the others are k_sparsity_rows_warp's
    const unsigned lights = __ballot_sync(0xffffffffu, light);
    if (__popc(lights) < kThreadMinLanes) {
      // too few light nodes to keep this warp's lanes busy (the boundary of a
      // dense mesh): they go to the warp kernel's list
      int base = 0;
      if (lane == 0 && lights) base = atomicAdd(defer_count, __popc(lights));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (light) defer[base + __popc(lights & ((1u << lane) - 1u))] = n;
      continue;
    }
    if (!light) continue;
    int D = 0;   // distinct neighbours; above DMAX the row is deferred
    bool bad = false;
    {
      CellStream<NPC> cs;
      cs.start(cn, nc_cell, nullptr, vec, b, e);
      for (int32_t p = b; p < e && D <= DMAX; ++p) {
        int32_t v[NPC];
        cs.next(cn, nc_cell, nullptr, vec, p, e, v);
#pragma unroll
        for (int j = 0; j < NPC; ++j) {
          const int32_t x = v[j];
          if (x == n) continue;
          if ((unsigned)x >= (unsigned)nb_node) {
            bad = true;
            continue;
          }
          // the table never holds more than DMAX < TS keys: the probe meets x or an empty slot
          int h = tab_hash(x) & (TS - 1);
#pragma unroll 1
          for (int q = 0; q < TS; ++q, h = (h + 1) & (TS - 1)) {
            const int32_t k = s_key[h][t];
            if (k == x) break;
            if (k == -1) {
              if (D < DMAX) {
                s_key[h][t] = x;
                s_at[D][t] = (uint8_t)h;
              }
              ++D;
              break;
            }
          }
        }
      }
    }
    const int stored = min(D, DMAX);
    if (bad) {
      atomicOr(err, 8);
      if (!FILL) row_len[n] = 0;
    } else if (D > DMAX) {
      defer_node(n, defer, defer_count);
    } else if (!FILL) {
      row_len[n] = D + 1;
    } else {
      // row_ptr null: the row goes to its padded place (afem_sparsity_rows)
      int64_t rb = (int64_t)(NPC - 1) * b + n;
      bool ok = true;
      if (row_ptr) {
        rb = __ldg(row_ptr + n);
        ok = __ldg(row_ptr + n + 1) - (int32_t)rb == D + 1;
        if (!ok) atomicOr(err, 4);
      } else {
        row_len[n] = D + 1;
      }
      if (ok) {
        int own = 0;   // neighbours below n
        if (D <= M && small_ids) {
          uint32_t a[M];
#pragma unroll
          for (int i = 0; i < M; ++i)
            a[i] = i < D ? ((uint32_t)s_key[s_at[i][t]][t] << SB) | (uint32_t)i : 0xffffffffu;
          bitonic_sort<M>(a);
#pragma unroll
          for (int i = 0; i < M; ++i) {
            if (i < D) {
              const int32_t x = (int32_t)(a[i] >> SB);
              const int pos = self_last ? i : i + (n < x);
              cols[rb + pos] = x;
              s_pos[s_at[a[i] & (M - 1)][t]][t] = (uint8_t)pos;
              own += x < n;
            }
          }
        } else {
          for (int i = 0; i < D; ++i) {
            const int32_t x = s_key[s_at[i][t]][t];
            int r = 0;
            for (int u = 0; u < D; ++u) r += s_key[s_at[u][t]][t] < x;
            const int pos = self_last ? r : r + (n < x);
            cols[rb + pos] = x;
            s_pos[s_at[i][t]][t] = (uint8_t)pos;
            own += x < n;
          }
        }
        const int pn = self_last ? D : own;
        cols[rb + pn] = n;
        CellStream<NPC> cs;
        cs.start(cn, nc_cell, nc_local, vec, b, e);
        for (int32_t p = b; p < e; ++p) {
          int32_t v[NPC];
          int li = cs.next(cn, nc_cell, nc_local, vec, p, e, v);
          if (!nc_local) li = local_index<NPC>(v, n, err);
          using Word = typename std::conditional<(NPC > 4), uint64_t, uint32_t>::type;
          Word word = (Word)pn;
#pragma unroll
          for (int j = 0; j < NPC; ++j) {
            if (j == li) continue;
            const int32_t x = v[j];
            Word q = (Word)pn;
            if (x != n) {
              int h = tab_hash(x) & (TS - 1);
#pragma unroll 1
              for (int k = 0; k < TS && s_key[h][t] != x; ++k) h = (h + 1) & (TS - 1);
              q = (Word)s_pos[h][t];
            }
            word |= q << (8 * (j < li ? j + 1 : j));
          }
          uint8_t* dst = slot + (int64_t)p * NPC;
          if (NPC == 4 && packed_slots) {
            *reinterpret_cast<uint32_t*>(dst) = (uint32_t)word;
          } else if (NPC == 8 && packed_slots) {
            *reinterpret_cast<uint2*>(dst) = make_uint2((uint32_t)word, (uint32_t)((uint64_t)word >> 32));
          } else {
#pragma unroll
            for (int q = 0; q < NPC; ++q) dst[q] = (uint8_t)((uint64_t)word >> (8 * q));
          }
        }
      }
    }
    // empty the table for the next node
    for (int i = 0; i < stored; ++i) s_key[s_at[i][t]][t] = -1;
  }
}

// The nodes in more than `min_deg` cells (every node when -1, none when
// INT_MAX), and the rows k_sparsity_thread or k_sparsity_rows_sub deferred
// (more distinct neighbours than their tables hold), listed
// in `list[0 .. *list_count)`: one warp per node, lanes over its incidences
// (chunks of 32).  The row's own node is inserted into the warp's hash set
// first, then every lane inserts the nodes of its cell: a node met again
// (the row's own included) finds its slot, so the number of first insertions
// D is the row length (the reference's deg + 1 entries,
// femutils/BSRFormat.cc:445-557).  Round r inserts, in every lane, the cell
// node r + 1 places after the lane's own, so that the lanes of one atomic
// rarely target the same slot (cells around a node share nodes at equal
// local indices).  With FILL the row is then written: the rank of each
// column among the row's (counted against the list with broadcast reads of
// shared memory; no sort) gives its position in either order, and every
// incidence writes its NPC slot bytes in one packed store.  Errors as
// k_sparsity_thread.
template <int NPC, bool FILL>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_sparsity_rows_warp(int nb_node, int min_deg, const int32_t* __restrict__ list,
                         const int32_t* __restrict__ list_count,
                         const int32_t* __restrict__ cn, const int32_t* __restrict__ nc_ptr,
                         const int32_t* __restrict__ nc_cell, const uint8_t* __restrict__ nc_local,
                         const int32_t* __restrict__ row_ptr, int self_last, int packed_slots,
                         int32_t* __restrict__ row_len, int32_t* __restrict__ cols, uint8_t* __restrict__ slot,
                         int* __restrict__ err) {
  __shared__ int32_t s_key[kWarpsPerBlock][kTabSlots];
  __shared__ int16_t s_at[kWarpsPerBlock][kTabSlots];
  __shared__ __align__(16) int32_t s_val[kWarpsPerBlock][FILL ? kTabSlots + 4 : 1];
  __shared__ uint8_t s_pos[kWarpsPerBlock][FILL ? kTabSlots : 1];
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int w = threadIdx.x >> 5;
  RowTables t{s_key[w], s_at[w], s_val[w], s_pos[w]};
  for (int i = lane; i < kTabSlots; i += 32) t.key[i] = -1;
  __syncwarp();
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const bool vec = (reinterpret_cast<uintptr_t>(cn) & 15) == 0;
  const int direct = min_deg == INT_MAX ? 0 : nb_node;   // INT_MAX: the list alone
  const int count = direct + *list_count;
  for (int it = wid; it < count; it += nwarps) {
    const int n = it < direct ? it : __ldg(list + (it - direct));
    const int32_t b = __ldg(nc_ptr + n);
    const int deg = __ldg(nc_ptr + n + 1) - b;
    if (it < direct && deg <= min_deg) continue;   // k_sparsity_thread's
    if (lane == 0) {
      const int h = tab_hash(n);
      t.key[h] = n;
      t.at[0] = (int16_t)h;
      if (FILL) t.val[0] = n;
    }
    __syncwarp();
    int32_t v[NPC];
    int16_t hs[NPC - 1];   // table slot of each round's candidate (the last chunk's)
    int li = 0;            // local index of n in the lane's cell
    bool act = false, bad = false, full = false;
    int D = 1;             // distinct columns so far, uniform across the warp
    for (int kb = 0; kb < deg; kb += 32) {
      act = kb + lane < deg;
      if (act) {
        load_cell<NPC>(cn, vec, __ldg(nc_cell + b + kb + lane), v);
        if (FILL && nc_local) {
          li = __ldg(nc_local + b + kb + lane);
        } else if (FILL) {
          li = local_index<NPC>(v, n, err);
        } else {
          li = 0;
#pragma unroll
          for (int j = NPC - 1; j > 0; --j)
            if (v[j] == n) li = j;
        }
#pragma unroll
        for (int j = 0; j < NPC; ++j) bad |= (unsigned)v[j] >= (unsigned)nb_node;
      }
#pragma unroll
      for (int r = 0; r + 1 < NPC; ++r) {
        int j = li + 1 + r;
        j -= j >= NPC ? NPC : 0;
        const int32_t x = pick<NPC>(v, j);
        bool fresh = false;
        int h = 0;
        if (act) {
          // one atomic settles the common case (an empty slot, or x already there);
          // a slot held by another node sends the lane on to the probing loop
          h = tab_hash(x);
          const int32_t old = atomicCAS(t.key + h, -1, x);
          fresh = old == -1;
          if (!fresh && old != x) {
            h = tab_insert(t.key, x, fresh);
            full |= h < 0;
          }
        }
        hs[r] = (int16_t)h;
        const unsigned fb = __ballot_sync(0xffffffffu, fresh);
        if (fresh) {
          const int at = D + __popc(fb & below);   // < kTabSlots: each first insertion took a table slot
          t.at[at] = (int16_t)h;
          if (FILL) t.val[at] = x;
        }
        D += __popc(fb);
      }
    }
    const bool bad_w = __any_sync(0xffffffffu, bad), overflow = __any_sync(0xffffffffu, full);
    const bool too_long = overflow || D > kMaxRowLen;
    __syncwarp();
    if (!FILL) {
      if (lane == 0) {
        if (bad_w || too_long) atomicOr(err, bad_w ? 8 : 2);
        row_len[n] = (bad_w || too_long) ? 0 : D;
      }
    } else {
      // row_ptr null: the row goes to its padded place (afem_sparsity_rows)
      const int64_t rb = row_ptr ? (int64_t)__ldg(row_ptr + n) : (int64_t)(NPC - 1) * b + n;
      const bool ok = !bad_w && !too_long && (!row_ptr || __ldg(row_ptr + n + 1) - (int32_t)rb == D);
      if (lane == 0 && !ok) atomicOr(err, bad_w ? 8 : too_long ? 2 : 4);
      if (lane == 0 && !row_ptr) row_len[n] = ok ? D : 0;
      if (ok) {
        if (lane < 4) t.val[D + lane] = INT_MAX;
        if (lane >= D && lane < 16) t.val[lane] = INT_MAX;
        __syncwarp();
        for (int i = lane; i < D; i += 32) {
          const int32_t x = t.val[i];
          int r = 0;
          if (D <= 16) {   // tetrahedral rows (15 entries): four broadcast reads, no loop
#pragma unroll
            for (int u = 0; u < 16; u += 4) {
              const int4 q = *reinterpret_cast<const int4*>(t.val + u);
              r += (q.x < x) + (q.y < x) + (q.z < x) + (q.w < x);
            }
          } else {
            for (int u = 0; u < D; u += 4) {
              const int4 q = *reinterpret_cast<const int4*>(t.val + u);
              r += (q.x < x) + (q.y < x) + (q.z < x) + (q.w < x);
            }
          }
          // self-last: the neighbours keep their ascending order, the row's own node goes last
          const int p = !self_last ? r : (x == n ? D - 1 : r - (x > n));
          cols[rb + p] = x;
          t.pos[t.at[i]] = (uint8_t)p;
        }
        __syncwarp();
        const int pn = t.pos[t.at[0]];
        for (int kb = 0; kb < deg; kb += 32) {
          if (deg > 32) {
            act = kb + lane < deg;
            if (act) {
              load_cell<NPC>(cn, vec, __ldg(nc_cell + b + kb + lane), v);
              li = nc_local ? __ldg(nc_local + b + kb + lane) : local_index<NPC>(v, n, err);
            }
          }
          if (!act) continue;
          // slot byte q of the incidence at bits 8q: its own column, then the
          // other cell nodes in increasing local index
          using Word = typename std::conditional<(NPC > 4), uint64_t, uint32_t>::type;
          Word word = (Word)pn;
#pragma unroll
          for (int r = 0; r + 1 < NPC; ++r) {
            int j = li + 1 + r;
            j -= j >= NPC ? NPC : 0;
            const Word p = (Word)t.pos[deg > 32 ? tab_find(t.key, pick<NPC>(v, j)) : hs[r]];
            word |= p << (8 * (j < li ? j + 1 : j));
          }
          uint8_t* dst = slot + (int64_t)(b + kb + lane) * NPC;
          if (NPC == 4 && packed_slots) {
            *reinterpret_cast<uint32_t*>(dst) = (uint32_t)word;
          } else if (NPC == 8 && packed_slots) {
            *reinterpret_cast<uint2*>(dst) = make_uint2((uint32_t)word, (uint32_t)((uint64_t)word >> 32));
          } else {
#pragma unroll
            for (int q = 0; q < NPC; ++q) dst[q] = (uint8_t)((uint64_t)word >> (8 * q));
          }
        }
      }
    }
    __syncwarp();
    for (int i = lane; i < D && i < kTabSlots; i += 32) t.key[t.at[i]] = -1;
    __syncwarp();
  }
}

// Dense meshes (tetrahedra, about 24 cells per node): a warp per 32 / G
// nodes, G lanes per node over its incidences in chunks of G, so that the
// lanes stay busy (24 incidences fill 3 chunks of 8 exactly, where a whole
// warp per node leaves 8 of its 32 lanes idle) and each node's fixed costs
// and ranking are shared by the warp's nodes.  The same hash sets as
// k_sparsity_rows_warp, one of SubTable::slots keys per node; the same
// rounds, ranks and slot bytes.  Nodes in more than 4 G cells, or with more
// than 3/4 of a table's slots in distinct neighbours, go to
// k_sparsity_rows_warp through the node list.  Errors as k_sparsity_thread.
constexpr int kSubLanes = 8;   // lanes per node of k_sparsity_rows_sub

template <int G>
struct SubTable {
  static constexpr int slots = G == 16 ? 256 : 128;
  static constexpr int bits = G == 16 ? 8 : 7;
  static constexpr int max_d = slots * 3 / 4;
  static constexpr int max_deg = 4 * G;
};

// Whether the insertion's table slots (one byte per round) and the local
// index fit one 32-bit word per chunk: three rounds (tetrahedra).
template <int NPC>
constexpr bool kKeepSlots = NPC <= 4;

template <int TS, int BITS>
__device__ __forceinline__ int sub_hash(int32_t v) { return (int)(((uint32_t)v * 2654435761u) >> (32 - BITS)); }

template <int NPC, bool FILL, int G>
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    k_sparsity_rows_sub(int nb_node, const int32_t* __restrict__ cn, const int32_t* __restrict__ nc_ptr,
                        const int32_t* __restrict__ nc_cell, const uint8_t* __restrict__ nc_local,
                        const int32_t* __restrict__ row_ptr, int self_last, int packed_slots,
                        int32_t* __restrict__ row_len, int32_t* __restrict__ cols, uint8_t* __restrict__ slot,
                        int32_t* __restrict__ defer, int32_t* __restrict__ defer_count, int* __restrict__ err) {
  using ST = SubTable<G>;
  constexpr int NG = 32 / G, TS = ST::slots, BITS = ST::bits, DMAX = ST::max_d;
  __shared__ int32_t s_key[kWarpsPerBlock][NG][TS];
  __shared__ int16_t s_at[kWarpsPerBlock][NG][DMAX];
  __shared__ __align__(16) int32_t s_val[kWarpsPerBlock][NG][FILL ? DMAX + 4 : 4];
  __shared__ uint8_t s_pos[kWarpsPerBlock][NG][FILL ? TS : 1];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int g = lane / G, gl = lane - g * G;
  const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << (g * G);
  const unsigned gbelow = gmask & ((1u << lane) - 1u);
  int32_t* const key = s_key[w][g];
  int16_t* const at = s_at[w][g];
  int32_t* const val = s_val[w][g];
  uint8_t* const pos = s_pos[w][g];
  for (int i = gl; i < TS; i += G) key[i] = -1;
  __syncwarp();
  const bool vec = (reinterpret_cast<uintptr_t>(cn) & 15) == 0;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int ngroups = (nb_node + NG - 1) / NG;
  for (int grp = wid; grp < ngroups; grp += nwarps) {
    const int n = grp * NG + g;
    int32_t b = 0;
    int deg = 0;
    if (n < nb_node) {
      b = __ldg(nc_ptr + n);
      deg = __ldg(nc_ptr + n + 1) - b;
    }
    const bool heavy = n < nb_node && deg > ST::max_deg;
    if (heavy && gl == 0) defer_node(n, defer, defer_count);
    const bool mine = n < nb_node && !heavy;
    if (mine && gl == 0) {
      const int h = sub_hash<TS, BITS>(n);
      key[h] = n;
      at[0] = (int16_t)h;
      if (FILL) val[0] = n;
    }
    __syncwarp();
    const int maxdeg = __reduce_max_sync(0xffffffffu, mine ? deg : 0);
    int D = 1;   // distinct columns so far, uniform across the node's lanes
    bool bad = false, full = false;
    // per chunk (at most 4: a node here has at most 4 G incidences), the
    // table slot of each round's candidate and the local index, one byte
    // each, for the slot bytes below (tetrahedra: 3 rounds)
    uint32_t kept[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int kb = c * G;
      if (kb >= maxdeg) break;
      const bool act = mine && kb + gl < deg;
      int32_t v[NPC];
      int li = 0;
      if (act) {
        load_cell<NPC>(cn, vec, __ldg(nc_cell + b + kb + gl), v);
        if (FILL && nc_local) {
          li = __ldg(nc_local + b + kb + gl);
        } else if (FILL) {
          li = local_index<NPC>(v, n, err);
        } else {
#pragma unroll
          for (int j = NPC - 1; j > 0; --j)
            if (v[j] == n) li = j;
        }
#pragma unroll
        for (int j = 0; j < NPC; ++j) bad |= (unsigned)v[j] >= (unsigned)nb_node;
      }
#pragma unroll
      for (int r = 0; r + 1 < NPC; ++r) {
        int j = li + 1 + r;
        j -= j >= NPC ? NPC : 0;
        bool fresh = false;
        int h = 0;
        if (act) {
          const int32_t x = pick<NPC>(v, j);
          h = sub_hash<TS, BITS>(x);
          const int32_t old = atomicCAS(key + h, -1, x);
          fresh = old == -1;
          if (!fresh && old != x) {
            h = -1;
#pragma unroll 1
            for (int p = 1; p < TS; ++p) {
              const int hp = (sub_hash<TS, BITS>(x) + p) & (TS - 1);
              const int32_t o = atomicCAS(key + hp, -1, x);
              if (o == -1 || o == x) {
                fresh = o == -1;
                h = hp;
                break;
              }
            }
            full |= h < 0;
          }
        }
        const unsigned fb = __ballot_sync(0xffffffffu, fresh);
        if (fresh) {
          const int a = D + __popc(fb & gbelow);
          if (a < DMAX) {
            at[a] = (int16_t)h;
            if (FILL) val[a] = pick<NPC>(v, j);
          } else {
            full = true;
          }
        }
        D += __popc(fb & gmask);
        if (kKeepSlots<NPC>) kept[c] |= (uint32_t)(h & 0xff) << (8 * r);
      }
      if (kKeepSlots<NPC>) kept[c] |= (uint32_t)li << 24;
    }
    const unsigned badm = __ballot_sync(0xffffffffu, bad), fullm = __ballot_sync(0xffffffffu, full);
    const bool bad_g = (badm & gmask) != 0;
    const bool spill = (fullm & gmask) != 0 || D > DMAX;   // keys past the slot list: clear the whole table
    const bool over_g = mine && !bad_g && spill;
    if (over_g && gl == 0) defer_node(n, defer, defer_count);
    if (!FILL) {
      if (mine && gl == 0) {
        if (bad_g) atomicOr(err, 8);
        if (bad_g || !over_g) row_len[n] = bad_g ? 0 : D;
      }
    } else {
      bool ok = mine && !bad_g && !over_g;
      int64_t rb = (int64_t)(NPC - 1) * b + n;
      if (mine && bad_g && gl == 0) atomicOr(err, 8);
      if (ok) {
        if (row_ptr) {
          rb = __ldg(row_ptr + n);
          ok = __ldg(row_ptr + n + 1) - (int32_t)rb == D;
          if (!ok && gl == 0) atomicOr(err, 4);
        } else if (gl == 0) {
          row_len[n] = D;
        }
      }
      if (ok)
        for (int i = D + gl; i < max(D + 4, 16); i += G) val[i] = INT_MAX;
      __syncwarp();
      if (ok) {
        for (int i = gl; i < D; i += G) {
          const int32_t x = val[i];
          int r = 0;
          if (D <= 16) {
#pragma unroll
            for (int u = 0; u < 16; u += 4) {
              const int4 q = *reinterpret_cast<const int4*>(val + u);
              r += (q.x < x) + (q.y < x) + (q.z < x) + (q.w < x);
            }
          } else {
            for (int u = 0; u < D; u += 4) {
              const int4 q = *reinterpret_cast<const int4*>(val + u);
              r += (q.x < x) + (q.y < x) + (q.z < x) + (q.w < x);
            }
          }
          // self-last: the neighbours keep their ascending order, the row's own node goes last
          const int p = !self_last ? r : (x == n ? D - 1 : r - (x > n));
          cols[rb + p] = x;
          pos[at[i]] = (uint8_t)p;
        }
      }
      __syncwarp();
      const int pn = ok ? pos[at[0]] : 0;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int kb = c * G;
        if (kb >= maxdeg) break;
        if (!ok || kb + gl >= deg) continue;
        // slot byte q of the incidence at bits 8q: its own column, then the
        // other cell nodes in increasing local index
        using Word = typename std::conditional<(NPC > 4), uint64_t, uint32_t>::type;
        Word word = (Word)pn;
        if constexpr (kKeepSlots<NPC>) {
          const int li = (int)(kept[c] >> 24);
#pragma unroll
          for (int r = 0; r + 1 < NPC; ++r) {
            int j = li + 1 + r;
            j -= j >= NPC ? NPC : 0;
            word |= (Word)pos[(kept[c] >> (8 * r)) & 0xffu] << (8 * (j < li ? j + 1 : j));
          }
        } else {
          int32_t v[NPC];
          load_cell<NPC>(cn, vec, __ldg(nc_cell + b + kb + gl), v);
          const int li = nc_local ? __ldg(nc_local + b + kb + gl) : local_index<NPC>(v, n, err);
#pragma unroll
          for (int r = 0; r + 1 < NPC; ++r) {
            int j = li + 1 + r;
            j -= j >= NPC ? NPC : 0;
            const int32_t x = pick<NPC>(v, j);
            int h = sub_hash<TS, BITS>(x);
#pragma unroll 1
            for (int q = 0; q < TS && key[h] != x; ++q) h = (h + 1) & (TS - 1);
            word |= (Word)pos[h] << (8 * (j < li ? j + 1 : j));
          }
        }
        uint8_t* dst = slot + (int64_t)(b + kb + gl) * NPC;
        if (NPC == 4 && packed_slots) {
          *reinterpret_cast<uint32_t*>(dst) = (uint32_t)word;
        } else if (NPC == 8 && packed_slots) {
          *reinterpret_cast<uint2*>(dst) = make_uint2((uint32_t)word, (uint32_t)((uint64_t)word >> 32));
        } else {
#pragma unroll
          for (int q = 0; q < NPC; ++q) dst[q] = (uint8_t)((uint64_t)word >> (8 * q));
        }
      }
    }
    __syncwarp();
    // empty the table: the recorded slots, or all of it after an overflow
    if (spill) {
      for (int i = gl; i < TS; i += G) key[i] = -1;
    } else if (mine) {
      for (int i = gl; i < D; i += G) key[at[i]] = -1;
    }
    __syncwarp();
  }
}

// Block CSR -> scalar CSR structure (BSRMatrix::toCsr, femutils/BSRFormat.cc:110-172).
__global__ void k_bsr_rows(int nb_brow, int b, const int32_t* __restrict__ brow_ptr, int32_t* __restrict__ row_ptr) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r <= nb_brow * b; r += gridDim.x * blockDim.x) {
    if (r == nb_brow * b) {
      row_ptr[r] = brow_ptr[nb_brow] * b * b;
      continue;
    }
    int br = r / b, i = r - br * b;
    int32_t s = brow_ptr[br], len = brow_ptr[br + 1] - s;
    row_ptr[r] = s * b * b + i * len * b;
  }
}

// The scalar columns of block row br fill one contiguous range,
// [s b^2, (s + len) b^2) with s = brow_ptr[br]: entry idx of it is scalar row
// i = idx / (len b), block x, component k.  A warp per block row writes the
// range with consecutive lanes on consecutive entries.
__global__ void k_bsr_cols(int nb_brow, int b, const int32_t* __restrict__ brow_ptr, const int32_t* __restrict__ bcols,
                           int32_t* __restrict__ cols) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t br = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; br < nb_brow; br += nwarps) {
    const int32_t s = __ldg(brow_ptr + br), len = __ldg(brow_ptr + br + 1) - s;
    const int row_len = len * b, total = row_len * b;
    int32_t* out = cols + (int64_t)s * b * b;
    for (int idx = lane; idx < total; idx += 32) {
      const int rem = idx % row_len;   // position within scalar row idx / row_len
      const int x = rem / b, k = rem - x * b;
      out[idx] = __ldg(bcols + s + x) * b + k;
    }
  }
}

}  // namespace afem

using namespace afem;

extern "C" {

afem_status afem_node_cell_build(afem_context ctx, int nb_node, int nb_cell, int npc, const int32_t* cell_nodes_d,
                                 int32_t* nc_ptr_d, int32_t* nc_cell_d, uint8_t* nc_local_d, int32_t* nc_inverse_d) {
  AFEM_CHECK_ARG(ctx, "afem_node_cell_build: null context");
  AFEM_CHECK_ARG(nb_node > 0 && nb_cell > 0, "afem_node_cell_build: empty mesh (nb_node=%d nb_cell=%d)", nb_node,
                 nb_cell);
  AFEM_CHECK_ARG(npc >= 2 && npc <= 8 && npc != 5 && npc != 6 && npc != 7,
                 "afem_node_cell_build: nodes_per_cell must be 2, 3, 4 or 8 (got %d)", npc);
  AFEM_CHECK_ARG(nb_cell < (1 << 28), "afem_node_cell_build: too many cells (%d)", nb_cell);
  AFEM_CHECK_ARG(cell_nodes_d && nc_ptr_d && nc_cell_d && nc_local_d, "afem_node_cell_build: null buffer");
  int64_t total = (int64_t)nb_cell * npc;
  AFEM_CHECK_ARG(total < INT_MAX, "afem_node_cell_build: too many incidences");
  size_t need = align256(sizeof(int32_t) * ((size_t)nb_node + 1)) + 2 * align256(sizeof(int32_t) * total) + 256 +
                scan_scratch_bytes(nb_node);
  AFEM_TRY(scratch_reserve(ctx, need));
  int32_t *cnt, *rank, *key;
  int* err;
  AFEM_TRY(scratch_take(ctx, (size_t)nb_node + 1, &cnt));
  AFEM_TRY(scratch_take(ctx, (size_t)total, &rank));
  AFEM_TRY(scratch_take(ctx, (size_t)total, &key));
  AFEM_TRY(scratch_take(ctx, 1, &err));
  AFEM_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ((size_t)nb_node + 1), ctx->stream));
  AFEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  AFEM_TRY(launch(ctx, k_nc_count, grid_for(ctx, total, 256), 256, 0, cell_nodes_d, total, nb_node, cnt, rank, err));
  AFEM_TRY(exclusive_scan_i32(ctx, cnt, nc_ptr_d, nb_node));
  AFEM_TRY(launch(ctx, k_nc_scatter, grid_for(ctx, total, 256), 256, 0, cell_nodes_d, total, npc, nb_node,
                  (const int32_t*)nc_ptr_d, (const int32_t*)rank, key));
  // measured at 128^3 tetrahedra (24 cells per node): warp 0.37 ms, thread 0.77 ms (its per-thread
  // stores are uncoalesced); Hexa8 96^3 and triangles 1024^2: the thread sort is the faster
  if (total > (int64_t)16 * nb_node)
    AFEM_TRY(launch(ctx, k_nc_sort_warp, grid_for(ctx, (int64_t)nb_node * 32, kWarpsPerBlock * 32, 8),
                    kWarpsPerBlock * 32, 0, nb_node, npc, (const int32_t*)nc_ptr_d, key, nc_cell_d, nc_local_d,
                    nc_inverse_d));
  else
    AFEM_TRY(launch(ctx, k_nc_sort_thread, grid_for(ctx, nb_node, 128), 128, 0, nb_node, npc,
                    (const int32_t*)nc_ptr_d, key, nc_cell_d, nc_local_d, nc_inverse_d));
  int herr = 0;
  AFEM_TRY(read_scalar(ctx, err, &herr));
  if (herr) return fail(AFEM_ERR_MESH, "afem_node_cell_build: node id out of range [0, %d) in cell_nodes", nb_node);
  return AFEM_OK;
}

}  // extern "C"

namespace afem {

// Resident blocks of a kernel on one SM: the grid-stride kernels below are
// launched with exactly that many blocks per SM, since a larger grid leaves
// its last blocks to a second, mostly idle wave.
template <typename Kernel>
static int resident_blocks(Kernel k, int block) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, block, 0) != cudaSuccess) {
    (void)cudaGetLastError();
    b = 0;
  }
  return b > 0 ? b : 1;
}

template <int NPC, bool FILL>
static afem_status launch_rows(afem_context ctx, bool dense, int nb_node, const int32_t* cn, const int32_t* nc_ptr,
                               const int32_t* nc_cell, const uint8_t* nc_local, const int32_t* row_ptr, int self_last,
                               int packed, int32_t* row_len, int32_t* cols, uint8_t* slot, int32_t* defer,
                               int32_t* defer_count, int* err) {
  static const int per_sm_thread = resident_blocks(k_sparsity_thread<NPC, FILL>, kThreadBlock);
  static const int per_sm_warp = resident_blocks(k_sparsity_rows_warp<NPC, FILL>, kWarpsPerBlock * 32);
  static const int per_sm_sub = resident_blocks(k_sparsity_rows_sub<NPC, FILL, kSubLanes>, kWarpsPerBlock * 32);
  if (!dense) {
    const unsigned g1 = (unsigned)std::min<int64_t>((nb_node + kThreadBlock - 1) / kThreadBlock,
                                                    (int64_t)ctx->sm_count * per_sm_thread);
    AFEM_TRY(launch(ctx, k_sparsity_thread<NPC, FILL>, g1, kThreadBlock, 0, nb_node, cn, nc_ptr, nc_cell, nc_local,
                    row_ptr, self_last, packed, row_len, cols, slot, defer, defer_count, err));
  } else {
    const int64_t groups = ((int64_t)nb_node + 32 / kSubLanes - 1) / (32 / kSubLanes);
    const unsigned g1 = (unsigned)std::min<int64_t>((groups + kWarpsPerBlock - 1) / kWarpsPerBlock,
                                                    (int64_t)ctx->sm_count * per_sm_sub);
    AFEM_TRY(launch(ctx, k_sparsity_rows_sub<NPC, FILL, kSubLanes>, g1, kWarpsPerBlock * 32, 0, nb_node, cn, nc_ptr,
                    nc_cell, nc_local, row_ptr, self_last, packed, row_len, cols, slot, defer, defer_count, err));
  }
  // the rows the thread or sub-warp kernel passed on (and, after the thread
  // kernel, the heavy ones): the grid covers the worst case and each warp
  // reads the list's length on the device
  const unsigned g2 = (unsigned)std::min<int64_t>((nb_node + kWarpsPerBlock - 1) / kWarpsPerBlock,
                                                  (int64_t)ctx->sm_count * per_sm_warp);
  return launch(ctx, k_sparsity_rows_warp<NPC, FILL>, g2, kWarpsPerBlock * 32, 0, nb_node,
                dense ? INT_MAX : ThreadTable<NPC>::max_deg, (const int32_t*)defer, (const int32_t*)defer_count, cn,
                nc_ptr, nc_cell, nc_local, row_ptr, self_last, packed, row_len, cols, slot, err);
}

static afem_status launch_sparsity_rows(afem_context ctx, bool fill, int nb_node, int npc, int64_t incidences,
                                        const int32_t* cn, const int32_t* nc_ptr, const int32_t* nc_cell,
                                        const uint8_t* nc_local, const int32_t* row_ptr, int self_last,
                                        int32_t* row_len, int32_t* cols, uint8_t* slot, int32_t* defer,
                                        int32_t* defer_count, int* err) {
  // Meshes whose nodes lie on average in more cells than the thread kernel
  // takes (tetrahedra: about 24) run the warp kernel alone: in the thread
  // kernel their few light nodes would only leave its lanes idle.
  const int max_deg = npc == 3 ? ThreadTable<3>::max_deg : npc == 4 ? ThreadTable<4>::max_deg : ThreadTable<8>::max_deg;
  const bool dense = incidences > (int64_t)max_deg * nb_node;
  // one packed store per incidence when the slot map is aligned to its rows
  const int packed = (reinterpret_cast<uintptr_t>(slot) % (npc == 8 ? 8 : 4)) == 0;
#define AFEM_ROWS_LAUNCH(NPC)                                                                                    \
  return fill ? launch_rows<NPC, true>(ctx, dense, nb_node, cn, nc_ptr, nc_cell, nc_local, row_ptr, self_last,     \
                                       packed, row_len, cols, slot, defer, defer_count, err)                      \
              : launch_rows<NPC, false>(ctx, dense, nb_node, cn, nc_ptr, nc_cell, nc_local, row_ptr, self_last,    \
                                        packed, row_len, cols, slot, defer, defer_count, err)
  if (npc == 3) AFEM_ROWS_LAUNCH(3);
  if (npc == 4) AFEM_ROWS_LAUNCH(4);
  AFEM_ROWS_LAUNCH(8);
#undef AFEM_ROWS_LAUNCH
}

// afem_sparsity_cols after afem_sparsity_rows on the same mesh: each row,
// found ascending at its padded offset, copied into place (self-last: the
// row's own node moved to the end and its slot bytes renumbered to match).
// Error bit 4: a row_ptr that does not match.
// One thread per node (rows of ~7 to ~15 entries: triangles, tetrahedra).
// With n16 > 0 (ascending order, both slot maps 16-byte aligned) the same
// launch also copies the slot map's first n16 16-byte chunks.
template <int NPC>
__global__ void k_sparsity_place_thread(int nb_node, const int32_t* __restrict__ nc_ptr,
                                        const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ pcols,
                                        const int32_t* __restrict__ plen, const uint8_t* __restrict__ pslot,
                                        int self_last, int32_t* __restrict__ cols, uint8_t* __restrict__ slot,
                                        int* __restrict__ err, int64_t n16) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += (int64_t)gridDim.x * blockDim.x)
    reinterpret_cast<int4*>(slot)[i] = __ldg(reinterpret_cast<const int4*>(pslot) + i);
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nb_node; n += gridDim.x * blockDim.x) {
    const int32_t rb = __ldg(row_ptr + n);
    const int len = __ldg(row_ptr + n + 1) - rb;
    if (len != __ldg(plen + n)) {
      atomicOr(err, 4);
      continue;
    }
    const int32_t b = __ldg(nc_ptr + n);
    const int32_t* src = pcols + (int64_t)(NPC - 1) * b + n;
    if (!self_last) {
      for (int i = 0; i < len; ++i) cols[rb + i] = __ldg(src + i);
      continue;
    }
    int pn = 0;   // the node's own position in the ascending row
    for (int i = 0; i < len; ++i)
      if (__ldg(src + i) == n) pn = i;
    for (int i = 0; i < len; ++i) cols[rb + (i == pn ? len - 1 : i - (i > pn))] = __ldg(src + i);
    const int32_t e = __ldg(nc_ptr + n + 1);
    for (int64_t q = (int64_t)NPC * b; q < (int64_t)NPC * e; ++q) {
      const int v = __ldg(pslot + q);
      slot[q] = (uint8_t)(v == pn ? len - 1 : v - (v > pn));
    }
  }
}

// A warp per 32 consecutive nodes, their rows copied one at a time across
// the lanes so that reads and writes move in contiguous segments (hexahedra:
// rows of ~27 entries, 64 slot bytes per incidence).
template <int NPC>
__global__ void k_sparsity_place_warp(int nb_node, const int32_t* __restrict__ nc_ptr, const int32_t* __restrict__ row_ptr,
                                      const int32_t* __restrict__ pcols, const int32_t* __restrict__ plen,
                                      const uint8_t* __restrict__ pslot, int self_last, int32_t* __restrict__ cols,
                                      uint8_t* __restrict__ slot, int* __restrict__ err, int64_t n16) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += (int64_t)gridDim.x * blockDim.x)
    reinterpret_cast<int4*>(slot)[i] = __ldg(reinterpret_cast<const int4*>(pslot) + i);
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t base = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * 32; base < nb_node;
       base += nwarps * 32) {
    const int n = (int)base + lane;
    int32_t rb = 0, b = 0, e = 0;
    int len = 0;
    if (n < nb_node) {
      rb = __ldg(row_ptr + n);
      len = __ldg(row_ptr + n + 1) - rb;
      b = __ldg(nc_ptr + n);
      e = __ldg(nc_ptr + n + 1);
      if (len != __ldg(plen + n)) {
        atomicOr(err, 4);
        len = 0;
      }
    }
    const int64_t src = (int64_t)(NPC - 1) * b + n;
    const int rows = min(32, nb_node - (int)base);
    for (int t = 0; t < rows; ++t) {
      const int32_t rbt = __shfl_sync(0xffffffffu, rb, t);
      const int lent = __shfl_sync(0xffffffffu, len, t);
      const int64_t st = __shfl_sync(0xffffffffu, src, t);
      if (!self_last) {
        for (int i = lane; i < lent; i += 32) cols[rbt + i] = __ldg(pcols + st + i);
        continue;
      }
      const int nt = (int)base + t;
      int pn = 0;   // the node's own position in its ascending row
      for (int i0 = 0; i0 < lent; i0 += 32) {
        const unsigned hit = __ballot_sync(0xffffffffu, i0 + lane < lent && __ldg(pcols + st + i0 + lane) == nt);
        if (hit) pn = i0 + __ffs(hit) - 1;
      }
      for (int i = lane; i < lent; i += 32) cols[rbt + (i == pn ? lent - 1 : i - (i > pn))] = __ldg(pcols + st + i);
      const int64_t q0 = (int64_t)NPC * __shfl_sync(0xffffffffu, b, t);
      const int64_t q1 = lent ? (int64_t)NPC * __shfl_sync(0xffffffffu, e, t) : q0;
      for (int64_t q = q0 + lane; q < q1; q += 32) {
        const int v = __ldg(pslot + q);
        slot[q] = (uint8_t)(v == pn ? lent - 1 : v - (v > pn));
      }
    }
  }
}

static afem_status sparsity_error(int herr, const char* fn) {
  if (herr & 8) return fail(AFEM_ERR_MESH, "%s: node id out of range in cell_nodes", fn);
  if (herr & 2)
    return fail(AFEM_ERR_MESH, "%s: a row has more than %d entries (%d neighbours)", fn, kMaxRowLen, kMaxRowLen - 1);
  return fail(AFEM_ERR_MESH, "%s: row_ptr does not match the mesh", fn);
}

}  // namespace afem

extern "C" {

afem_status afem_sparsity_rows(afem_context ctx, int nb_node, int npc, const int32_t* cell_nodes_d,
                               const int32_t* nc_ptr_d, const int32_t* nc_cell_d, int32_t* row_ptr_d, int64_t* nnz_h) {
  AFEM_CHECK_ARG(ctx, "afem_sparsity_rows: null context");
  AFEM_CHECK_ARG(nb_node > 0 && (npc == 3 || npc == 4 || npc == 8), "afem_sparsity_rows: bad sizes");
  AFEM_CHECK_ARG(cell_nodes_d && nc_ptr_d && nc_cell_d && row_ptr_d, "afem_sparsity_rows: null buffer");
  size_t need = 2 * align256(sizeof(int32_t) * ((size_t)nb_node + 1)) + 256 + scan_scratch_bytes(nb_node);
  AFEM_TRY(scratch_reserve(ctx, need));
  int32_t *len, *defer;
  int* err;   // err[0] error bits, err[1] deferred rows
  AFEM_TRY(scratch_take(ctx, (size_t)nb_node + 1, &len));
  AFEM_TRY(scratch_take(ctx, (size_t)nb_node + 1, &defer));
  AFEM_TRY(scratch_take(ctx, 2, &err));
  int32_t incidences = 0;
  AFEM_TRY(read_scalar(ctx, nc_ptr_d + nb_node, &incidences));
  AFEM_CUDA(cudaMemsetAsync(err, 0, 2 * sizeof(int), ctx->stream));
  // The whole rows (columns and slot map) in one pass, kept for
  // afem_sparsity_cols, when the device has room for them; else the row
  // lengths alone and afem_sparsity_cols finds the rows again.
  auto& sp = ctx->sp;
  sp.valid = false;
  const size_t pcols = (size_t)(npc - 1) * incidences + nb_node;
  const size_t bytes = align256(sizeof(int32_t) * pcols) + align256(sizeof(int32_t) * ((size_t)nb_node + 1)) +
                       align256((size_t)npc * incidences);
  if (bytes > sp.cap) {   // grows, kept until the context goes
    if (sp.buf) AFEM_CUDA(cudaFreeAsync(sp.buf, ctx->stream));
    sp.buf = nullptr;
    sp.cap = 0;
    if (cudaMallocAsync(&sp.buf, bytes, ctx->stream) == cudaSuccess) {
      sp.cap = bytes;
    } else {
      (void)cudaGetLastError();
      sp.buf = nullptr;
    }
  }
  if (sp.buf) {
    char* q = static_cast<char*>(sp.buf);
    sp.cols = reinterpret_cast<int32_t*>(q);
    sp.len = reinterpret_cast<int32_t*>(q + align256(sizeof(int32_t) * pcols));
    sp.slot = reinterpret_cast<uint8_t*>(q + align256(sizeof(int32_t) * pcols) +
                                         align256(sizeof(int32_t) * ((size_t)nb_node + 1)));
    AFEM_TRY(launch_sparsity_rows(ctx, true, nb_node, npc, incidences, cell_nodes_d, nc_ptr_d, nc_cell_d, nullptr,
                                  nullptr, 0, sp.len, sp.cols, sp.slot, defer, err + 1, err));
    AFEM_TRY(exclusive_scan_i32(ctx, sp.len, row_ptr_d, nb_node));
  } else {
    AFEM_TRY(launch_sparsity_rows(ctx, false, nb_node, npc, incidences, cell_nodes_d, nc_ptr_d, nc_cell_d, nullptr,
                                  nullptr, 0, len, nullptr, nullptr, defer, err + 1, err));
    AFEM_TRY(exclusive_scan_i32(ctx, len, row_ptr_d, nb_node));
  }
  // the error bits and the total in one read-back
  int32_t* hb = reinterpret_cast<int32_t*>(ctx->pinned);
  AFEM_CUDA(cudaMemcpyAsync(hb, err, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  AFEM_CUDA(cudaMemcpyAsync(hb + 1, row_ptr_d + nb_node, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
  const int herr = hb[0];
  if (herr & ~16) return sparsity_error(herr, "afem_sparsity_rows");
  if (sp.buf) {
    // a cell holding a node twice (bit 16): its slot bytes need the node -> cell local indices
    sp.valid = (herr & 16) == 0;
    sp.cn = cell_nodes_d;
    sp.nc_ptr = nc_ptr_d;
    sp.nc_cell = nc_cell_d;
    sp.nb_node = nb_node;
    sp.npc = npc;
    sp.incidences = incidences;
  }
  if (nnz_h) *nnz_h = hb[1];
  return AFEM_OK;
}

afem_status afem_sparsity_cols(afem_context ctx, int nb_node, int npc, const int32_t* cell_nodes_d,
                               const int32_t* nc_ptr_d, const int32_t* nc_cell_d, const uint8_t* nc_local_d,
                               const int32_t* row_ptr_d, int col_order, int32_t* cols_d, uint8_t* nc_slot_d) {
  AFEM_CHECK_ARG(ctx, "afem_sparsity_cols: null context");
  AFEM_CHECK_ARG(nb_node > 0 && (npc == 3 || npc == 4 || npc == 8), "afem_sparsity_cols: bad sizes");
  AFEM_CHECK_ARG(col_order == AFEM_COLS_ASCENDING || col_order == AFEM_COLS_SELF_LAST,
                 "afem_sparsity_cols: bad col_order %d", col_order);
  AFEM_CHECK_ARG(cell_nodes_d && nc_ptr_d && nc_cell_d && nc_local_d && row_ptr_d && cols_d && nc_slot_d,
                 "afem_sparsity_cols: null buffer");
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(int32_t) * ((size_t)nb_node + 1)) + 256));
  int32_t* defer;
  int* err;   // err[0] error bits, err[1] deferred rows
  AFEM_TRY(scratch_take(ctx, (size_t)nb_node + 1, &defer));
  AFEM_TRY(scratch_take(ctx, 2, &err));
  AFEM_CUDA(cudaMemsetAsync(err, 0, 2 * sizeof(int), ctx->stream));
  auto& sp = ctx->sp;
  const bool self_last = col_order == AFEM_COLS_SELF_LAST;
  if (sp.buf && sp.valid && sp.cn == cell_nodes_d && sp.nc_ptr == nc_ptr_d && sp.nc_cell == nc_cell_d &&
      sp.nb_node == nb_node && sp.npc == npc) {
    // the rows afem_sparsity_rows found on these mesh arrays, copied into place
    auto kern = npc == 3 ? k_sparsity_place_thread<3> : npc == 4 ? k_sparsity_place_thread<4> : k_sparsity_place_warp<8>;
    // ascending order: the slot map is copied as it is, by the thread-per-node
    // launch when aligned (measured: 2D 0.071 -> 0.062 ms; the hexahedral
    // warp copy is faster beside a separate copy of its 64-byte slot words)
    const size_t sbytes = (size_t)npc * sp.incidences;
    const int64_t n16 =
        (!self_last && npc != 8 && ((uintptr_t)nc_slot_d & 15) == 0) ? (int64_t)(sbytes / 16) : 0;
    AFEM_TRY(launch(ctx, kern, grid_for(ctx, (int64_t)nb_node, 256), 256, 0, nb_node, nc_ptr_d, row_ptr_d,
                    (const int32_t*)sp.cols, (const int32_t*)sp.len, (const uint8_t*)sp.slot, (int)self_last,
                    cols_d, nc_slot_d, err, n16));
    if (!self_last && sbytes > (size_t)n16 * 16)
      AFEM_CUDA(cudaMemcpyAsync(nc_slot_d + n16 * 16, sp.slot + n16 * 16, sbytes - (size_t)n16 * 16,
                                cudaMemcpyDeviceToDevice, ctx->stream));
    sp.valid = false;
  } else {
    int32_t incidences = 0;
    AFEM_TRY(read_scalar(ctx, nc_ptr_d + nb_node, &incidences));
    AFEM_TRY(launch_sparsity_rows(ctx, true, nb_node, npc, incidences, cell_nodes_d, nc_ptr_d, nc_cell_d, nc_local_d,
                                  row_ptr_d, (int)self_last, nullptr, cols_d, nc_slot_d, defer, err + 1, err));
  }
  int herr = 0;
  AFEM_TRY(read_scalar(ctx, err, &herr));
  if (herr) return sparsity_error(herr, "afem_sparsity_cols");
  return AFEM_OK;
}

afem_status afem_bsr_to_csr_structure(afem_context ctx, int nb_brow, int b, const int32_t* brow_ptr_d,
                                      const int32_t* bcols_d, int32_t* row_ptr_d, int32_t* cols_d) {
  AFEM_CHECK_ARG(ctx && nb_brow > 0 && b >= 1 && b <= 8, "afem_bsr_to_csr_structure: bad arguments");
  AFEM_CHECK_ARG(brow_ptr_d && bcols_d && row_ptr_d && cols_d, "afem_bsr_to_csr_structure: null buffer");
  scratch_reset(ctx);
  AFEM_TRY(launch(ctx, k_bsr_rows, grid_for(ctx, (int64_t)nb_brow * b + 1, 256), 256, 0, nb_brow, b, brow_ptr_d,
                  row_ptr_d));
  return launch(ctx, k_bsr_cols, grid_for(ctx, (int64_t)nb_brow * 32, 256), 256, 0, nb_brow, b, brow_ptr_d, bcols_d,
                cols_d);
}

}  // extern "C"
