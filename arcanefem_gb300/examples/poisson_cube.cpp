// C++ host path over the C ABI (include/afem_gb300.hpp), the way an Arcane
// module's compute() drives the reference (modules/poisson/FemModule.cc:75-146):
// initialize -> computeSparsity -> assembleBilinear -> toLinearSystem ->
// source term -> Dirichlet -> applyLinearSystemTransformationAndSolve.
//
//   poisson_cube <n> <solution.bin>
//
// Unit cube, n^3 hexahedra split in 6 tetrahedra (no jitter), f = 1,
// u = 0 on x = 0 and x = 1 (row-column elimination), Jacobi CG to 1e-10.
// Writes the nodal solution (float64) and prints one line of results.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "afem_gb300.hpp"

int main(int argc, char** argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 8;
  const char* out = argc > 2 ? argv[2] : nullptr;
  const int m = n + 1;
  const int nb_node = m * m * m, nb_cell = 6 * n * n * n;
  std::vector<double> coords(3 * (size_t)nb_node);
  for (int k = 0; k < m; ++k)
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        size_t id = i + (size_t)m * (j + (size_t)m * k);
        coords[3 * id] = (double)i / n;
        coords[3 * id + 1] = (double)j / n;
        coords[3 * id + 2] = (double)k / n;
      }
  // the 6 Kuhn tetrahedra of a hexahedron (corner = dx + 2 dy + 4 dz), positive volume
  const int kuhn[6][4] = {{0, 1, 3, 7}, {0, 5, 1, 7}, {0, 3, 2, 7}, {0, 2, 6, 7}, {0, 4, 5, 7}, {0, 6, 4, 7}};
  std::vector<int32_t> cells(4 * (size_t)nb_cell);
  std::vector<int32_t> dir;
  size_t c = 0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        int32_t corner[8];
        for (int q = 0; q < 8; ++q)
          corner[q] = (i + (q & 1)) + m * ((j + ((q >> 1) & 1)) + m * (k + ((q >> 2) & 1)));
        for (int t = 0; t < 6; ++t, ++c)
          for (int v = 0; v < 4; ++v) cells[4 * c + v] = corner[kuhn[t][v]];
      }
  for (int k = 0; k < m; ++k)
    for (int j = 0; j < m; ++j) {
      dir.push_back(0 + m * (j + m * k));
      dir.push_back(n + m * (j + m * k));
    }
  try {
    cudaStream_t s;
    afem::check_cuda(cudaStreamCreate(&s), "cudaStreamCreate");
    afem::Context ctx(s);
    afem::DeviceArray<double> d_coords(coords.size(), s);
    afem::DeviceArray<int32_t> d_cells(cells.size(), s), d_dir(dir.size(), s);
    afem::check_cuda(cudaMemcpyAsync(d_coords.data(), coords.data(), coords.size() * 8, cudaMemcpyHostToDevice, s), "h2d");
    afem::check_cuda(cudaMemcpyAsync(d_cells.data(), cells.data(), cells.size() * 4, cudaMemcpyHostToDevice, s), "h2d");
    afem::check_cuda(cudaMemcpyAsync(d_dir.data(), dir.data(), dir.size() * 4, cudaMemcpyHostToDevice, s), "h2d");

    afem::MeshView mesh{3, nb_node, nb_cell, d_coords.data(), d_cells.data()};
    afem::BSRFormat fmt(ctx, mesh);
    fmt.initialize(1, true);
    fmt.computeSparsity();
    fmt.assemblePoisson();
    afem::CsrDoFLinearSystem ls(ctx, nb_node);
    fmt.toLinearSystem(ls);
    fmt.applyConstantSourceToRhs(1.0, ls.rhsVariable());
    ls.applyDirichletViaElimination(AFEM_ELIMINATE_ROW_COLUMN, d_dir.data(), (int)dir.size(), 1, 0, 0.0);
    ls.applyMatrixTransformation();
    ls.applyRHSTransformation();
    afem_solver_options opt;
    afem_solver_options_default(&opt);
    opt.rtol = 1e-10;
    opt.max_iter = 10000;
    afem_solve_info info = ls.solve(&opt);
    // the reference's CSR impl throws on eliminateRow: so does this one
    bool threw = false;
    try {
      ls.eliminateRow(0, 1.0);
    } catch (const afem::Error& e) {
      threw = e.status() == AFEM_ERR_NOT_IMPLEMENTED;
    }
    std::vector<double> u(nb_node);
    afem::check_cuda(cudaMemcpyAsync(u.data(), ls.solutionVariable(), u.size() * 8, cudaMemcpyDeviceToHost, s), "d2h");
    afem::check_cuda(cudaStreamSynchronize(s), "sync");
    if (out) {
      FILE* f = std::fopen(out, "wb");
      if (!f || std::fwrite(u.data(), 8, u.size(), f) != u.size()) throw afem::Error(AFEM_ERR_BAD_ARG, "write failed");
      std::fclose(f);
    }
    std::printf("nodes=%d cells=%d nnz=%lld iterations=%d relres=%.3e eliminate_row_throws=%d\n", nb_node, nb_cell,
                (long long)fmt.nbNonZeroBlocks(), info.iterations, info.relres, threw ? 1 : 0);
    return (info.status == AFEM_OK && threw) ? 0 : 1;
  } catch (const afem::Error& e) {
    std::fprintf(stderr, "afem error %d: %s\n", e.status(), e.what());
    return 2;
  }
}
