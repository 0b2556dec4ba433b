// Drives the GB300 linear-system service (arcanefem_gb300/arcane/
// GB300DoFLinearSystem.cc) through the IDoFLinearSystemImpl interface, as a
// module would: a reference CSR view with unused (-1) slots on the device,
// DoF flags in the Arcane variables, applyMatrixTransformation,
// applyRHSTransformation, solve; then clearValues and the same sequence again
// on fresh values (a second solve).  Test infrastructure.
//
//   adapter_driver <input dir> <output dir>
// inputs: meta.txt ("n nb_column precision"), rows.i32 [n], cols.i32
// [nb_column], vals.f64 [nb_column], rhs.f64, forced_info.u8,
// forced_value.f64, elim_info.u8, elim_value.f64 [n];
// outputs: values{1,2}.f64 (transformed), rhs{1,2}.f64 (transformed),
// sol{1,2}.f64, info.txt.
#include <GB300DoFLinearSystem.h>
#include <IDoFLinearSystemFactory.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

using namespace Arcane;
using namespace Arcane::FemUtils;

template <class T>
static std::vector<T> load(const std::string& path, size_t n)
{
  std::vector<T> v(n);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
  if (!f)
    throw std::runtime_error("cannot read " + path);
  return v;
}

template <class T>
static void save(const std::string& path, const T* p, size_t n)
{
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(p), (std::streamsize)(n * sizeof(T)));
}

template <class T>
static T* to_device(const std::vector<T>& v)
{
  T* d = nullptr;
  if (cudaMalloc(&d, v.size() * sizeof(T)) != cudaSuccess ||
      cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    throw std::runtime_error("device copy failed");
  return d;
}

int main(int argc, char** argv)
{
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s <input dir> <output dir>\n", argv[0]);
    return 2;
  }
  const std::string in = argv[1], out = argv[2];
  int n = 0, precision = 0;
  long long nb_column = 0;
  {
    std::ifstream m(in + "/meta.txt");
    m >> n >> nb_column >> precision;
  }
  auto rows = load<Int32>(in + "/rows.i32", n);
  auto cols = load<Int32>(in + "/cols.i32", nb_column);
  auto vals = load<Real>(in + "/vals.f64", nb_column);
  auto rhs = load<Real>(in + "/rhs.f64", n);
  auto finfo = load<unsigned char>(in + "/forced_info.u8", n);
  auto fval = load<Real>(in + "/forced_value.f64", n);
  auto einfo = load<unsigned char>(in + "/elim_info.u8", n);
  auto eval = load<Real>(in + "/elim_value.f64", n);

  // the view's arrays live on the device, as the reference's accelerator path keeps them
  Int32* rows_d = to_device(rows);
  Int32* cols_d = to_device(cols);
  Real* vals_d = to_device(vals);
  std::vector<Int32> counts(n);   // nbColumnForRow: the range size, as CsrFormat stores it
  for (int i = 0; i < n; ++i)
    counts[i] = (i + 1 < n ? rows[i + 1] : (Int32)nb_column) - rows[i];
  auto view = CSRFormatView::make(SmallSpan<const Int32>(rows_d, n), SmallSpan<const Int32>(counts.data(), n),
                                  SmallSpan<const Int32>(cols_d, nb_column), SmallSpan<Real>(vals_d, nb_column));

  IItemFamily dofs(n);
  afem_solver_options opt;
  afem_solver_options_default(&opt);
  opt.rtol = 1e-10;
  opt.max_iter = 20000;
  opt.precision = precision;
  opt.skip_forced_rows = 1;   // penalty rows (1e30 diagonals) stay out of the stop test
  std::unique_ptr<IDoFLinearSystemImpl> ls(createGB300DoFLinearSystemImpl(&dofs, "Poisson", opt, nullptr));
  auto* gb = static_cast<GB300DoFLinearSystemImpl*>(ls.get());
  std::ofstream info(out + "/info.txt");

  // the CSR implementation's unsupported calls throw, as the reference's do
  try {
    ls->eliminateRow(DoFLocalId(0), 1.0);
    info << "eliminateRow did_not_throw\n";
  }
  catch (const NotImplementedException&) {
    info << "eliminateRow NotImplementedException\n";
  }

  for (int pass = 1; pass <= 2; ++pass) {
    if (pass == 2) {
      // fresh values (the transformation changed them in place), flags reset, view set again
      cudaMemcpy(vals_d, vals.data(), vals.size() * sizeof(Real), cudaMemcpyHostToDevice);
      ls->clearValues();
    }
    for (int i = 0; i < n; ++i) {
      ls->rhsVariable()[DoFLocalId(i)] = rhs[i];
      ls->solutionVariable()[DoFLocalId(i)] = 0.0;
      ls->getForcedInfo()[DoFLocalId(i)] = finfo[i] != 0;
      ls->getForcedValue()[DoFLocalId(i)] = fval[i];
      ls->getEliminationInfo()[DoFLocalId(i)] = einfo[i];
      ls->getEliminationValue()[DoFLocalId(i)] = eval[i];
    }
    ls->setCSRValues(view);
    if (pass == 1) {
      // an entry outside the sparsity is an error, one inside it is added in place
      try {
        ls->matrixAddValue(DoFLocalId(0), DoFLocalId(n - 1), 1.0);
        info << "matrixAddValue_outside did_not_throw\n";
      }
      catch (const FatalErrorException&) {
        info << "matrixAddValue_outside FatalErrorException\n";
      }
      ls->matrixAddValue(DoFLocalId(1), DoFLocalId(1), 0.0);
    }
    ls->applyMatrixTransformation();
    ls->applyRHSTransformation();
    ls->solve();
    const auto& si = gb->lastSolveInfo();
    info << "pass " << pass << " iterations " << si.iterations << " relres " << si.relres << " status " << si.status
         << "\n";
    std::vector<Real> tv(nb_column);
    cudaMemcpy(tv.data(), vals_d, tv.size() * sizeof(Real), cudaMemcpyDeviceToHost);
    save(out + "/values" + std::to_string(pass) + ".f64", tv.data(), tv.size());
    save(out + "/rhs" + std::to_string(pass) + ".f64", ls->rhsVariable().asArray().data(), n);
    save(out + "/sol" + std::to_string(pass) + ".f64", ls->solutionVariable().asArray().data(), n);
  }
  ls.reset();
  cudaFree(rows_d);
  cudaFree(cols_d);
  cudaFree(vals_d);
  info << "done\n";
  return 0;
}
