/*
 * afem_oracle_dok.cc -- the reference's CPU "DOK" assembly, restated for the
 * CPU baseline.  TEST INFRASTRUCTURE ONLY (a timed baseline and a checker,
 * never the product).
 *
 * modules/poisson/FemModule.cc:398-421 (_assembleBilinear): for every cell,
 * the element matrix K_e = vol (dxU ^ dxU) + vol (dyU ^ dyU) [+ vol (dzU ^ dzU)]
 * (modules/poisson/ElementMatrix.h:28-49,79-88), then matrixAddValue(row, col,
 * K_e(i, j)) for every pair of cell nodes.  The Aleph linear system skips
 * zero values and keeps an ordered map of (row, column) -> value with
 * insert-or-add (femutils/AlephDoFLinearSystem.cc:125-135,
 * femutils/internal/OrderedRowColumnMap.h:59-93); the map is then read in
 * order into CSR.  Built with -ffp-contract=off like the rest of the oracle.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <utility>

#include "afem_oracle.h"

namespace {

struct RowColumn {
  int32_t row, col;
  bool operator<(const RowColumn& o) const { return row == o.row ? col < o.col : row < o.row; }
};

// K_e row by row from the oracle's element vectors (the same gradients and
// measure as the module's CPU element matrix; its vol (dxU ^ dxU) + ... sums
// round differently in the last bits, which this timing baseline does not
// need to reproduce)
void element_matrix(int kind, const double* coords, const int32_t* cn, double K[4][4]) {
  if (kind == AFO_POISSON_TRI3) {
    double row[3];
    for (int i = 0; i < 3; ++i) {
      afo_elem_vec_poisson_tri3(coords, cn, i, row);
      for (int k = 0; k < 3; ++k) K[i][k] = row[k];
    }
    return;
  }
  double row[4];
  for (int i = 0; i < 4; ++i) {
    afo_elem_vec_poisson_tet4(coords, cn, i, row);
    for (int k = 0; k < 4; ++k) K[i][k] = row[k];
  }
}

}  // namespace

/* DOK assembly of cells [0, nb_cell): returns the number of stored entries
 * (zeros skipped) written to row_ptr[nb_node + 1], cols, values (capacity
 * cap), or -1 when cap is too small.  Poisson P1 triangles / tetrahedra. */
extern "C" int64_t afo_assemble_dok(int kind, int nb_node, int nb_cell, const double* coords,
                                    const int32_t* cell_nodes, int32_t* row_ptr, int32_t* cols, double* values,
                                    int64_t cap) {
  const int npc = kind == AFO_POISSON_TRI3 ? 3 : 4;
  std::map<RowColumn, double> map;
  double K[4][4];
  for (int c = 0; c < nb_cell; ++c) {
    const int32_t* cn = cell_nodes + (int64_t)c * npc;
    element_matrix(kind, coords, cn, K);
    for (int i = 0; i < npc; ++i)
      for (int j = 0; j < npc; ++j) {
        const double v = K[i][j];
        if (v == 0.0) continue;   // AlephDoFLinearSystem::matrixAddValue skips zeros
        RowColumn rc{cn[i], cn[j]};
        auto x = map.find(rc);
        if (x == map.end())
          map.insert(std::make_pair(rc, v));
        else
          x->second += v;
      }
  }
  const int64_t nnz = (int64_t)map.size();
  if (nnz > cap) return -1;
  std::memset(row_ptr, 0, sizeof(int32_t) * ((size_t)nb_node + 1));
  int64_t k = 0;
  for (const auto& e : map) {
    row_ptr[e.first.row + 1]++;
    cols[k] = e.first.col;
    values[k] = e.second;
    ++k;
  }
  for (int i = 0; i < nb_node; ++i) row_ptr[i + 1] += row_ptr[i];
  return nnz;
}
