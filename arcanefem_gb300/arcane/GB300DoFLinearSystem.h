// GB300DoFLinearSystem.h -- the GB300 linear-system back-end of ArcaneFEM.
//
// An IDoFLinearSystemImpl (femutils/internal/IDoFLinearSystemImpl.h:37-70)
// whose matrix transformations and Krylov solve run in libafem_gb300.so
// through its C ABI (include/afem_gb300.h).  It takes the reference's CSR
// view as the assembly leaves it (femutils/CsrFormatMatrixView.h:135-210:
// N row starts, the last row ending at nbColumn(), unused slots holding -1)
// with no repacking copy, and it keeps the reference's semantics:
//   - setCSRValues keeps a non-owning view valid until solve()
//     (femutils/DoFLinearSystem.h:318-328);
//   - eliminateRow / eliminateRowColumn throw NotImplementedException, as the
//     CSR implementation does (femutils/internal/CsrDoFLinearSystemImpl.h:67-75):
//     elimination goes through the DoF flag variables;
//   - applyMatrixTransformation may run again after clearValues, and solve()
//     may run more than once (modules/testlab/FemModule.cc:1988-2021).
// Options (GB300DoFLinearSystemFactory.axl): rtol, atol, max-iter, precond
// {jacobi, none, learned}, precision {fp64, mixed}, inner-rtol,
// skip-forced-rows, block-size.
//
// The file lives next to femutils/HypreDoFLinearSystem.cc in an ArcaneFEM
// build; its service registration (GB300DoFLinearSystem.cc) is compiled when
// ARCANEFEM_GB300_ARCANE_SERVICE is defined (the axl-generated base class
// exists there).
#ifndef ARCANEFEM_FEMUTILS_GB300DOFLINEARSYSTEM_H
#define ARCANEFEM_FEMUTILS_GB300DOFLINEARSYSTEM_H

#include "CsrFormatMatrixView.h"
#include "internal/DoFLinearSystemImplBase.h"

#include <afem_gb300.h>

namespace Arcane::FemUtils
{

class GB300DoFLinearSystemImpl
: public DoFLinearSystemImplBase
{
 public:

  //! cuda_stream: the stream of the module's RunQueue (nullptr: the legacy default stream).
  GB300DoFLinearSystemImpl(IItemFamily* dof_family, const String& solver_name, void* cuda_stream = nullptr);
  ~GB300DoFLinearSystemImpl() override;

 public:

  void matrixAddValue(DoFLocalId row, DoFLocalId column, Real value) override;
  void matrixSetValue(DoFLocalId row, DoFLocalId column, Real value) override;
  void eliminateRow(DoFLocalId row, Real value) override;
  void eliminateRowColumn(DoFLocalId row, Real value) override;
  void applyMatrixTransformation() override;
  void applyRHSTransformation() override;
  void solve() override;
  void setSolverCommandLineArguments(const CommandLineArguments&) override {}
  void clearValues() override;
  void setCSRValues(const CSRFormatView& csr_view) override;
  CSRFormatView& getCSRValues() override { return m_csr_view; }
  bool hasSetCSRValues() const override { return true; }

  // service options
  void setRelTolerance(Real v) { m_options.rtol = v; }
  void setAbsTolerance(Real v) { m_options.atol = v; }
  void setMaxIter(Int32 v) { m_options.max_iter = v; }
  void setPreconditioner(int precond) { m_options.precond = precond; }   // AFEM_PRECOND_*
  void setPrecision(int precision) { m_options.precision = precision; }  // AFEM_PRECISION_*
  void setInnerRelTolerance(Real v) { m_options.inner_rtol = v; }
  void setSkipForcedRows(bool v) { m_options.skip_forced_rows = v ? 1 : 0; }
  void setBlockSize(Int32 b) { m_options.block_size = b; }
  //! Element arithmetic of the library's assembly kernels on this context (AFEM_FORMULATION_*).
  void setElementFormulation(int f);

  //! The last solve's iterations, refinements, status and true FP64 relative residual.
  const afem_solve_info& lastSolveInfo() const { return m_info; }
  afem_context context() const { return m_ctx; }

 private:

  void _check(afem_status s, const char* what) const;
  void _ensureSystem();
  void _bindView();
  void _copyFlagsIn();
  void _copyIn(VariableDoFReal& v, double* device_array);
  void _copyOut(double* device_array, VariableDoFReal& v);
  void _synchronize();

  afem_context m_ctx = nullptr;
  afem_linear_system m_ls = nullptr;
  afem_solver_options m_options;
  afem_solve_info m_info{};
  CSRFormatView m_csr_view;
  bool m_view_bound = false;
};

//! createInstance of the service: what the factory service returns.
IDoFLinearSystemImpl* createGB300DoFLinearSystemImpl(IItemFamily* dof_family, const String& solver_name,
                                                     const afem_solver_options& options, void* cuda_stream);

} // namespace Arcane::FemUtils

#endif
