// Connectivity and sparsity for P1 meshes.
//
// node -> cell adjacency (the transpose of cell -> node):
//   histogram of incidences, exclusive scan, scatter, then a per-node
//   segmented sort of (cell, local) keys so that cells come out ascending --
//   the order of Arcane's nodeCell() connectivity.  The histogram and scatter
//   use integer atomics on per-node counters; the segmented sort (a bitonic
//   network in registers, one warp per node) makes the result independent of
//   their order, so the output is deterministic.
//
// node -> node sparsity (rows of the assembled matrix):
//   one warp per node inserts the nodes of its incident cells into a hash
//   table in shared memory; the number of distinct values is the row length
//   = 1 + number of neighbours (femutils/BSRFormat.cc:445-557, row = deg + 1).
//   The second pass sorts the distinct values and writes the columns
//   (ascending or self-last) and, for every cell-node incidence, its position
//   in the row (the slot map used by the assembly kernels).  Rows too long
//   for the table path extract their distinct values in increasing order by
//   warp-wide minima instead.
#include <algorithm>
#include <climits>

#include "afem_internal.cuh"

namespace afem {

// ---------------------------------------------------------------------------
// node -> cell

__global__ void k_nc_count(const int32_t* __restrict__ cn, int64_t total, int nb_node, int32_t* __restrict__ cnt,
                           int* __restrict__ err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t n = cn[i];
    if (n < 0 || n >= nb_node) {
      atomicOr(err, 1);
      continue;
    }
    atomicAdd(&cnt[n], 1);
  }
}

__global__ void k_nc_scatter(const int32_t* __restrict__ cn, int64_t total, int npc, int nb_node,
                             const int32_t* __restrict__ nc_ptr, int32_t* __restrict__ cursor,
                             int32_t* __restrict__ key) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    int32_t n = cn[i];
    if (n < 0 || n >= nb_node) continue;
    int32_t pos = nc_ptr[n] + atomicAdd(&cursor[n], 1);
    int32_t cell = (int32_t)(i / npc);
    int32_t local = (int32_t)(i - (int64_t)cell * npc);
    key[pos] = (cell << 3) | local;  // cells < 2^28 checked by the caller; local < 8
  }
}

constexpr int kWarpsPerBlock = 8;

// Per-node sort of the (cell << 3 | local) keys, then split; the inverse map
// records, for each (cell, local), its incidence index.  One warp per node:
// up to 32 keys are sorted by a bitonic network on registers (shuffles);
// longer lists (rare) by an insertion sort in lane 0.
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_nc_sort(int nb_node, int npc,
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

constexpr int kRowCap = 512;        // candidates per node (deg * npc), e.g. 128 tetrahedra
constexpr int kMaxRowLen = 255;     // slot map entries are uint8

// One warp per node.  The candidates (the nodes of the node's incident
// cells, m = deg * npc of them) are held in registers, R per lane (candidate
// i in lane i % 32, register i / 32), with, for the column pass, the slot-map
// index of each: k * npc + q for candidate i = cell node j of incidence
// k = i / npc, q = 0 for the row's own node (local index li) and q = 1.. for
// the other cell nodes in increasing local index -- the order of the element
// rows.  The distinct candidates come out in increasing order, one warp-wide
// minimum per distinct value; the sweep that finds value t + 1 also writes
// the slot bytes of value t, so each distinct value costs one sweep of R
// registers.  Returns the row length; with `fill`, writes the columns
// (ascending or self-last) at cols[0..len) and the slot map.
template <int R, bool FILL>
__device__ __forceinline__ int row_select(int n, int npc, int m, const int32_t* __restrict__ cn,
                                          const int32_t* __restrict__ nc_cell, const uint8_t* __restrict__ local,
                                          int len, int self_last, int32_t* __restrict__ cols,
                                          uint8_t* __restrict__ slot) {
  const int lane = threadIdx.x & 31;
  int32_t v[R];
  int16_t si[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int i = r * 32 + lane;
    v[r] = INT_MAX;
    si[r] = 0;
    if (i < m) {
      const int k = i / npc, j = i - k * npc;
      v[r] = __ldg(cn + (int64_t)__ldg(nc_cell + k) * npc + j);
      if (FILL) {
        const int li = __ldg(local + k);
        si[r] = (int16_t)(k * npc + (j == li ? 0 : (j < li ? j + 1 : j)));
      }
    }
  }
  int32_t last = INT_MIN;
  int pos_last = -1, it = 0;
  for (;;) {
    int32_t loc = INT_MAX;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (FILL && v[r] == last && pos_last >= 0) slot[si[r]] = (uint8_t)pos_last;
      if (v[r] > last && v[r] < loc) loc = v[r];
    }
    const int32_t mn = __reduce_min_sync(0xffffffffu, loc);
    if (mn == INT_MAX) break;
    if (FILL) {
      const int pos = self_last ? (mn < n ? it : (mn == n ? len - 1 : it - 1)) : it;
      // a row_ptr that disagrees is reported by the caller, not written past
      pos_last = (pos >= 0 && pos < len) ? pos : -1;
      if (lane == 0 && pos_last >= 0) cols[pos_last] = mn;
    }
    last = mn;
    ++it;
  }
  return it;
}

// Fast path for rows of at most kHashRow candidates and 32 distinct columns
// (every interior row of a tetrahedral, triangular or hexahedral mesh): each
// candidate is inserted once into a per-warp open-addressing table in shared
// memory (atomicCAS, linear probing), so the row length is the number of
// first insertions -- one pass over the candidates instead of one sweep per
// distinct value.  The column pass compacts the first insertions (ballot
// prefix) into a list, sorts it (one value per lane, a 32-key bitonic network
// on shuffles), records each value's position in the row in its table entry,
// and every candidate reads its slot byte from there.  Rows with more
// candidates, and column passes with more than 32 distinct values, take
// row_select.  Returns the row length, or -1 when the row needs row_select.
constexpr int kHashRow = 128;      // candidates per row on the fast path (R = 4)
constexpr int kHashSlots = 256;    // table entries per warp (load factor <= 1/8 for 32 distinct values)

__device__ __forceinline__ uint32_t hash_slot(int32_t v) { return ((uint32_t)v * 2654435761u) >> 24; }

template <bool FILL>
__device__ __forceinline__ int row_hash(int n, int npc, int m, const int32_t* __restrict__ cn,
                                        const int32_t* __restrict__ nc_cell, const uint8_t* __restrict__ local,
                                        int len, int self_last, int32_t* __restrict__ cols,
                                        uint8_t* __restrict__ slot, int32_t* __restrict__ key,
                                        uint8_t* __restrict__ rank, uint64_t* __restrict__ list) {
  constexpr int R = kHashRow / 32;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
#pragma unroll
  for (int k = lane; k < kHashSlots; k += 32) key[k] = -1;
  __syncwarp();
  int16_t si[R];
  int16_t hs[R];
  int distinct = 0;   // uniform across the warp
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int i = r * 32 + lane;
    si[r] = 0;
    hs[r] = 0;
    bool fresh = false;
    int32_t v = -1;
    if (i < m) {
      const int k = i / npc, j = i - k * npc;
      v = __ldg(cn + (int64_t)__ldg(nc_cell + k) * npc + j);
      if (FILL) {
        const int li = __ldg(local + k);
        si[r] = (int16_t)(k * npc + (j == li ? 0 : (j < li ? j + 1 : j)));
      }
      uint32_t h = hash_slot(v);
      for (int probe = 0; probe < kHashSlots; ++probe, h = (h + 1) & (kHashSlots - 1)) {
        const int32_t old = atomicCAS(key + h, -1, v);
        if (old == -1) {
          fresh = true;
          break;
        }
        if (old == v) break;
      }
      hs[r] = (int16_t)h;
    }
    const unsigned fb = __ballot_sync(0xffffffffu, fresh);
    if (FILL && fresh) {
      const int at = distinct + __popc(fb & below);
      if (at < 32) list[at] = ((uint64_t)(uint32_t)v << 32) | (uint32_t)hs[r];
    }
    distinct += __popc(fb);
  }
  if (!FILL) return distinct;   // the table counts any number of distinct values
  if (distinct > 32) return -1;
  __syncwarp();
  // the distinct values, one per lane, sorted by a 32-key bitonic network;
  // each carries its table slot
  uint64_t kv = lane < distinct ? list[lane] : ~uint64_t(0);
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const uint64_t o = __shfl_xor_sync(0xffffffffu, kv, j);
      const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
      kv = keep_min ? (o < kv ? o : kv) : (o > kv ? o : kv);
    }
  }
  // lane t < distinct now holds the t-th smallest column; a row_ptr that
  // disagrees is reported by the caller, not written past
  if (distinct == len) {
    if (lane < distinct) {
      const int32_t col = (int32_t)(kv >> 32);
      // self-last: the neighbours keep their ascending order, the row's own node goes last
      const int pos = !self_last ? lane : (col < n ? lane : (col == n ? len - 1 : lane - 1));
      cols[pos] = col;
      rank[(uint32_t)kv & 0xffffu] = (uint8_t)pos;
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (r * 32 + lane < m) slot[si[r]] = rank[hs[r]];
  }
  __syncwarp();
  return distinct;
}

template <bool FILL>
__device__ __forceinline__ int row_dispatch(int n, int npc, int m, const int32_t* cn, const int32_t* nc_cell,
                                            const uint8_t* local, int len, int self_last, int32_t* cols,
                                            uint8_t* slot, int32_t* key, uint8_t* rank, uint64_t* list) {
  if (m <= kHashRow) {
    const int got = row_hash<FILL>(n, npc, m, cn, nc_cell, local, len, self_last, cols, slot, key, rank, list);
    if (got >= 0) return got;
  }
  if (m <= 32) return row_select<1, FILL>(n, npc, m, cn, nc_cell, local, len, self_last, cols, slot);
  if (m <= 64) return row_select<2, FILL>(n, npc, m, cn, nc_cell, local, len, self_last, cols, slot);
  if (m <= 128) return row_select<4, FILL>(n, npc, m, cn, nc_cell, local, len, self_last, cols, slot);
  if (m <= 256) return row_select<8, FILL>(n, npc, m, cn, nc_cell, local, len, self_last, cols, slot);
  return row_select<16, FILL>(n, npc, m, cn, nc_cell, local, len, self_last, cols, slot);
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_row_len(int nb_node, int npc, const int32_t* __restrict__ cn,
                                                                 const int32_t* __restrict__ nc_ptr,
                                                                 const int32_t* __restrict__ nc_cell,
                                                                 int32_t* __restrict__ row_len,
                                                                 int* __restrict__ err) {
  __shared__ int32_t tab_key[kWarpsPerBlock][kHashSlots];
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  int32_t* const key = tab_key[threadIdx.x >> 5];
  for (int n = wid; n < nb_node; n += nwarps) {
    const int32_t b = __ldg(nc_ptr + n);
    const int m = (__ldg(nc_ptr + n + 1) - b) * npc;
    // a node in no cell keeps its diagonal (the reference's rows hold deg + 1 entries)
    int len = m > kRowCap ? -1
              : m == 0    ? 1
                          : row_dispatch<false>(n, npc, m, cn, nc_cell + b, nullptr, 0, 0, nullptr, nullptr, key,
                                                nullptr, nullptr);
    if (lane == 0) {
      if (len < 0 || len > kMaxRowLen) {
        atomicOr(err, 2);
        len = 0;
      }
      row_len[n] = len;
    }
  }
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_row_fill(int nb_node, int npc, const int32_t* __restrict__ cn,
                                                                  const int32_t* __restrict__ nc_ptr,
                                                                  const int32_t* __restrict__ nc_cell,
                                                                  const uint8_t* __restrict__ nc_local,
                                                                  const int32_t* __restrict__ row_ptr, int self_last,
                                                                  int32_t* __restrict__ cols,
                                                                  uint8_t* __restrict__ slot, int* __restrict__ err) {
  __shared__ int32_t tab_key[kWarpsPerBlock][kHashSlots];
  __shared__ uint8_t tab_rank[kWarpsPerBlock][kHashSlots];
  __shared__ uint64_t tab_list[kWarpsPerBlock][32];
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  int32_t* const key = tab_key[threadIdx.x >> 5];
  uint8_t* const rank = tab_rank[threadIdx.x >> 5];
  uint64_t* const list = tab_list[threadIdx.x >> 5];
  for (int n = wid; n < nb_node; n += nwarps) {
    const int32_t rb = __ldg(row_ptr + n);
    const int len = __ldg(row_ptr + n + 1) - rb;
    const int32_t b = __ldg(nc_ptr + n);
    const int m = (__ldg(nc_ptr + n + 1) - b) * npc;
    int got = -1;
    if (m == 0) {   // a node in no cell: its diagonal only
      got = 1;
      if (lane == 0 && len == 1) cols[rb] = n;
    } else if (m <= kRowCap) {
      got = row_dispatch<true>(n, npc, m, cn, nc_cell + b, nc_local + b, len, self_last, cols + rb,
                               slot + (int64_t)b * npc, key, rank, list);
    }
    if (lane == 0 && got != len) atomicOr(err, 4);
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

__global__ void k_bsr_cols(int nb_brow, int b, const int32_t* __restrict__ brow_ptr, const int32_t* __restrict__ bcols,
                           int32_t* __restrict__ cols) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nb_brow * b; r += gridDim.x * blockDim.x) {
    int br = r / b, i = r - br * b;
    int32_t s = brow_ptr[br], len = brow_ptr[br + 1] - s;
    int64_t o = (int64_t)s * b * b + (int64_t)i * len * b;
    for (int32_t x = 0; x < len; ++x)
      for (int k = 0; k < b; ++k) cols[o + (int64_t)x * b + k] = bcols[s + x] * b + k;
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
  size_t need = 2 * align256(sizeof(int32_t) * ((size_t)nb_node + 1)) + align256(sizeof(int32_t) * total) + 256 +
                scan_scratch_bytes(nb_node);
  AFEM_TRY(scratch_reserve(ctx, need));
  int32_t *cnt, *cursor, *key;
  int* err;
  AFEM_TRY(scratch_take(ctx, (size_t)nb_node + 1, &cnt));
  AFEM_TRY(scratch_take(ctx, (size_t)nb_node + 1, &cursor));
  AFEM_TRY(scratch_take(ctx, (size_t)total, &key));
  AFEM_TRY(scratch_take(ctx, 1, &err));
  AFEM_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ((size_t)nb_node + 1), ctx->stream));
  AFEM_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * ((size_t)nb_node + 1), ctx->stream));
  AFEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  AFEM_TRY(launch(ctx, k_nc_count, grid_for(ctx, total, 256), 256, 0, cell_nodes_d, total, nb_node, cnt, err));
  AFEM_TRY(exclusive_scan_i32(ctx, cnt, nc_ptr_d, nb_node));
  AFEM_TRY(launch(ctx, k_nc_scatter, grid_for(ctx, total, 256), 256, 0, cell_nodes_d, total, npc, nb_node,
                  (const int32_t*)nc_ptr_d, cursor, key));
  AFEM_TRY(launch(ctx, k_nc_sort, grid_for(ctx, (int64_t)nb_node * 32, kWarpsPerBlock * 32, 8), kWarpsPerBlock * 32, 0,
                  nb_node, npc, (const int32_t*)nc_ptr_d, key, nc_cell_d, nc_local_d, nc_inverse_d));
  int herr = 0;
  AFEM_TRY(read_scalar(ctx, err, &herr));
  if (herr) return fail(AFEM_ERR_MESH, "afem_node_cell_build: node id out of range [0, %d) in cell_nodes", nb_node);
  return AFEM_OK;
}

afem_status afem_sparsity_rows(afem_context ctx, int nb_node, int npc, const int32_t* cell_nodes_d,
                               const int32_t* nc_ptr_d, const int32_t* nc_cell_d, int32_t* row_ptr_d, int64_t* nnz_h) {
  AFEM_CHECK_ARG(ctx, "afem_sparsity_rows: null context");
  AFEM_CHECK_ARG(nb_node > 0 && (npc == 3 || npc == 4 || npc == 8), "afem_sparsity_rows: bad sizes");
  AFEM_CHECK_ARG(cell_nodes_d && nc_ptr_d && nc_cell_d && row_ptr_d, "afem_sparsity_rows: null buffer");
  size_t need = align256(sizeof(int32_t) * ((size_t)nb_node + 1)) + 256 + scan_scratch_bytes(nb_node);
  AFEM_TRY(scratch_reserve(ctx, need));
  int32_t* len;
  int* err;
  AFEM_TRY(scratch_take(ctx, (size_t)nb_node + 1, &len));
  AFEM_TRY(scratch_take(ctx, 1, &err));
  AFEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  unsigned grid =
      (unsigned)std::min<int64_t>((nb_node + kWarpsPerBlock - 1) / kWarpsPerBlock, (int64_t)ctx->sm_count * 8);
  AFEM_TRY(launch(ctx, k_row_len, grid, kWarpsPerBlock * 32, 0, nb_node, npc, cell_nodes_d, nc_ptr_d, nc_cell_d, len,
                  err));
  AFEM_TRY(exclusive_scan_i32(ctx, len, row_ptr_d, nb_node));
  int herr = 0;
  AFEM_TRY(read_scalar(ctx, err, &herr));
  if (herr)
    return fail(AFEM_ERR_MESH,
                "afem_sparsity_rows: a node has more than %d cell-node incidences or more than %d neighbours",
                kRowCap, kMaxRowLen);
  if (nnz_h) {
    int32_t nnz = 0;
    AFEM_TRY(read_scalar(ctx, row_ptr_d + nb_node, &nnz));
    *nnz_h = nnz;
  }
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
  AFEM_TRY(scratch_reserve(ctx, 256));
  int* err;
  AFEM_TRY(scratch_take(ctx, 1, &err));
  AFEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  unsigned grid =
      (unsigned)std::min<int64_t>((nb_node + kWarpsPerBlock - 1) / kWarpsPerBlock, (int64_t)ctx->sm_count * 8);
  AFEM_TRY(launch(ctx, k_row_fill, grid, kWarpsPerBlock * 32, 0, nb_node, npc, cell_nodes_d, nc_ptr_d, nc_cell_d,
                  nc_local_d, row_ptr_d, col_order, cols_d, nc_slot_d, err));
  int herr = 0;
  AFEM_TRY(read_scalar(ctx, err, &herr));
  if (herr) return fail(AFEM_ERR_MESH, "afem_sparsity_cols: row_ptr does not match the mesh");
  return AFEM_OK;
}

afem_status afem_bsr_to_csr_structure(afem_context ctx, int nb_brow, int b, const int32_t* brow_ptr_d,
                                      const int32_t* bcols_d, int32_t* row_ptr_d, int32_t* cols_d) {
  AFEM_CHECK_ARG(ctx && nb_brow > 0 && b >= 1 && b <= 8, "afem_bsr_to_csr_structure: bad arguments");
  AFEM_CHECK_ARG(brow_ptr_d && bcols_d && row_ptr_d && cols_d, "afem_bsr_to_csr_structure: null buffer");
  scratch_reset(ctx);
  AFEM_TRY(launch(ctx, k_bsr_rows, grid_for(ctx, (int64_t)nb_brow * b + 1, 256), 256, 0, nb_brow, b, brow_ptr_d,
                  row_ptr_d));
  return launch(ctx, k_bsr_cols, grid_for(ctx, (int64_t)nb_brow * b, 256), 256, 0, nb_brow, b, brow_ptr_d, bcols_d,
                cols_d);
}

}  // extern "C"
