// GB300DoFLinearSystem.cc -- IDoFLinearSystemImpl over libafem_gb300.so.
//
// The DoF variables stay Arcane's (DoFLinearSystemImplBase); the library keeps
// device copies, filled from them before each transformation / solve and
// copied back where the reference modifies them in place (the right-hand side
// in applyRHSTransformation, the solution in solve).  cudaMemcpyDefault lets
// the variables live in host, pinned or device memory.
#include "GB300DoFLinearSystem.h"

#include <arcane/utils/FatalErrorException.h>
#include <cuda_runtime.h>

#include <type_traits>

namespace Arcane::FemUtils
{

static_assert(sizeof(Bool) == sizeof(uint8_t) && sizeof(Byte) == sizeof(uint8_t),
              "the forced / elimination flags are one byte per DoF on both sides");
static_assert(std::is_same_v<Real, double>, "the library's values are IEEE double");

GB300DoFLinearSystemImpl::
GB300DoFLinearSystemImpl(IItemFamily* dof_family, const String& solver_name, void* cuda_stream)
: DoFLinearSystemImplBase(dof_family, solver_name)
{
  afem_solver_options_default(&m_options);
  _check(afem_context_create(&m_ctx, cuda_stream), "afem_context_create");
}

GB300DoFLinearSystemImpl::
~GB300DoFLinearSystemImpl()
{
  afem_ls_destroy(m_ls);
  afem_context_destroy(m_ctx);
}

void GB300DoFLinearSystemImpl::
_check(afem_status s, const char* what) const
{
  if (s == AFEM_OK)
    return;
  if (s == AFEM_ERR_NOT_IMPLEMENTED)
    ARCANE_THROW(NotImplementedException, "GB300 {0}: {1}", what, afem_last_error());
  if (s == AFEM_ERR_BAD_ARG)
    ARCANE_THROW(ArgumentException, "GB300 {0}: {1}", what, afem_last_error());
  ARCANE_FATAL("GB300 {0} (status {1}): {2}", what, s, afem_last_error());
}

void GB300DoFLinearSystemImpl::
setElementFormulation(int f)
{
  _check(afem_context_set_element_formulation(m_ctx, f), "afem_context_set_element_formulation");
}

void GB300DoFLinearSystemImpl::
_ensureSystem()
{
  if (!m_ls)
    _check(afem_ls_create(m_ctx, dofFamily()->nbItem(), &m_ls), "afem_ls_create");
}

void GB300DoFLinearSystemImpl::
setCSRValues(const CSRFormatView& csr_view)
{
  // non-owning, as CsrDoFLinearSystemImpl::setCSRValues; bound to the library on first use
  m_csr_view = csr_view;
  m_view_bound = false;
}

void GB300DoFLinearSystemImpl::
_bindView()
{
  _ensureSystem();
  if (m_view_bound)
    return;
  // rows(): the row starts without a trailing entry; the per-row count is the
  // row's range, which is what CsrFormat stores in nbColumnForRow
  // (femutils/CsrFormatMatrix.cc:76-95), hence no count array
  const CSRFormatView& v = m_csr_view;
  _check(afem_ls_set_csr_view(m_ls, v.nbRow(), v.rows().data(), nullptr, v.nbColumn(), v.columns().data(),
                              v.values().data()),
         "afem_ls_set_csr_view");
  m_view_bound = true;
}

void GB300DoFLinearSystemImpl::
_copyIn(VariableDoFReal& var, double* device_array)
{
  auto a = var.asArray();
  cudaError_t e = cudaMemcpy(device_array, a.data(), sizeof(double) * a.size(), cudaMemcpyDefault);
  if (e != cudaSuccess)
    ARCANE_FATAL("GB300 copy in: {0}", cudaGetErrorString(e));
}

void GB300DoFLinearSystemImpl::
_copyOut(double* device_array, VariableDoFReal& var)
{
  _synchronize();
  auto a = var.asArray();
  cudaError_t e = cudaMemcpy(a.data(), device_array, sizeof(double) * a.size(), cudaMemcpyDefault);
  if (e != cudaSuccess)
    ARCANE_FATAL("GB300 copy out: {0}", cudaGetErrorString(e));
}

void GB300DoFLinearSystemImpl::
_copyFlagsIn()
{
  double *rhs, *sol, *fv, *ev;
  uint8_t *fi, *ei;
  _check(afem_ls_dof_variables(m_ls, &rhs, &sol, &fi, &fv, &ei, &ev), "afem_ls_dof_variables");
  _synchronize();   // earlier library work on the device arrays is finished
  auto fia = getForcedInfo().asArray();
  auto eia = getEliminationInfo().asArray();
  cudaError_t e = cudaMemcpy(fi, fia.data(), fia.size(), cudaMemcpyDefault);
  if (e == cudaSuccess)
    e = cudaMemcpy(ei, eia.data(), eia.size(), cudaMemcpyDefault);
  if (e != cudaSuccess)
    ARCANE_FATAL("GB300 copy of the DoF flags: {0}", cudaGetErrorString(e));
  _copyIn(getForcedValue(), fv);
  _copyIn(getEliminationValue(), ev);
}

void GB300DoFLinearSystemImpl::
_synchronize()
{
  _check(afem_context_synchronize(m_ctx), "afem_context_synchronize");
}

void GB300DoFLinearSystemImpl::
matrixAddValue(DoFLocalId row, DoFLocalId column, Real value)
{
  _bindView();
  _check(afem_ls_matrix_add_value(m_ls, row.localId(), column.localId(), value), "matrixAddValue");
}

void GB300DoFLinearSystemImpl::
matrixSetValue(DoFLocalId row, DoFLocalId column, Real value)
{
  _bindView();
  _check(afem_ls_matrix_set_value(m_ls, row.localId(), column.localId(), value), "matrixSetValue");
}

void GB300DoFLinearSystemImpl::
eliminateRow(DoFLocalId, Real)
{
  ARCANE_THROW(NotImplementedException, "");
}

void GB300DoFLinearSystemImpl::
eliminateRowColumn(DoFLocalId, Real)
{
  ARCANE_THROW(NotImplementedException, "");
}

void GB300DoFLinearSystemImpl::
applyMatrixTransformation()
{
  _bindView();
  _copyFlagsIn();
  _check(afem_ls_apply_matrix_transformation(m_ls), "applyMatrixTransformation");
}

void GB300DoFLinearSystemImpl::
applyRHSTransformation()
{
  _bindView();
  double *rhs, *sol, *fv, *ev;
  uint8_t *fi, *ei;
  _check(afem_ls_dof_variables(m_ls, &rhs, &sol, &fi, &fv, &ei, &ev), "afem_ls_dof_variables");
  _synchronize();
  _copyIn(rhsVariable(), rhs);
  _check(afem_ls_apply_rhs_transformation(m_ls), "applyRHSTransformation");
  _copyOut(rhs, rhsVariable());
}

void GB300DoFLinearSystemImpl::
solve()
{
  _bindView();
  double *rhs, *sol, *fv, *ev;
  uint8_t *fi, *ei;
  _check(afem_ls_dof_variables(m_ls, &rhs, &sol, &fi, &fv, &ei, &ev), "afem_ls_dof_variables");
  _synchronize();
  _copyIn(rhsVariable(), rhs);
  _copyIn(solutionVariable(), sol);   // the initial guess
  // the forced rows, for skip-forced-rows
  auto fia = getForcedInfo().asArray();
  cudaError_t e = cudaMemcpy(fi, fia.data(), fia.size(), cudaMemcpyDefault);
  if (e != cudaSuccess)
    ARCANE_FATAL("GB300 copy of the forced flags: {0}", cudaGetErrorString(e));
  const afem_status s = afem_ls_solve(m_ls, &m_options, &m_info);
  _copyOut(sol, solutionVariable());
  _check(s, "solve");
}

void GB300DoFLinearSystemImpl::
clearValues()
{
  DoFLinearSystemImplBase::clearValues();
  if (m_ls)
    _check(afem_ls_clear_values(m_ls), "clearValues");
  m_view_bound = false;
}

IDoFLinearSystemImpl*
createGB300DoFLinearSystemImpl(IItemFamily* dof_family, const String& solver_name, const afem_solver_options& options,
                               void* cuda_stream)
{
  auto* x = new GB300DoFLinearSystemImpl(dof_family, solver_name, cuda_stream);
  x->setRelTolerance(options.rtol);
  x->setAbsTolerance(options.atol);
  x->setMaxIter(options.max_iter);
  x->setPreconditioner(options.precond);
  x->setPrecision(options.precision);
  x->setInnerRelTolerance(options.inner_rtol);
  x->setSkipForcedRows(options.skip_forced_rows != 0);
  x->setBlockSize(options.block_size);
  return x;
}

} // namespace Arcane::FemUtils

#ifdef ARCANEFEM_GB300_ARCANE_SERVICE
// The service, as femutils/HypreDoFLinearSystem.cc:863-898 registers HYPRE's:
// selected by <linear-system name="GB300LinearSystem"> (modules/*/Fem.axl).
#include "GB300DoFLinearSystemFactory_axl.h"

namespace Arcane::FemUtils
{

class GB300DoFLinearSystemFactoryService
: public ArcaneGB300DoFLinearSystemFactoryObject
{
 public:

  explicit GB300DoFLinearSystemFactoryService(const ServiceBuildInfo& sbi)
  : ArcaneGB300DoFLinearSystemFactoryObject(sbi)
  {}

  IDoFLinearSystemImpl*
  createInstance(ISubDomain*, IItemFamily* dof_family, const String& solver_name) override
  {
    afem_solver_options o;
    afem_solver_options_default(&o);
    o.rtol = options()->rtol();
    o.atol = options()->atol();
    o.max_iter = options()->maxIter();
    o.precond = options()->precond();
    o.precision = options()->precision();
    o.inner_rtol = options()->innerRtol();
    o.skip_forced_rows = options()->skipForcedRows() ? 1 : 0;
    o.block_size = options()->blockSize();
    return createGB300DoFLinearSystemImpl(dof_family, solver_name, o, nullptr);
  }
};

ARCANE_REGISTER_SERVICE_GB300DOFLINEARSYSTEMFACTORY(GB300LinearSystem, GB300DoFLinearSystemFactoryService);

} // namespace Arcane::FemUtils
#endif
