// Stand-in for femutils/internal/DoFLinearSystemImplBase.h: the DoF variables
// every implementation shares (rhs, solution, forced info / value,
// elimination info / value) and clearValues, which resets the flags as the
// reference's does (DoFLinearSystemImplBase.cc:44-50).
#pragma once
#include "IDoFLinearSystemImpl.h"

namespace Arcane::FemUtils
{
class DoFLinearSystemImplBase
: public TraceAccessor
, public IDoFLinearSystemImpl
{
 public:
  DoFLinearSystemImplBase(IItemFamily* dof_family, const String& solver_name)
  : TraceAccessor(dof_family->traceMng())
  , m_dof_family(dof_family)
  , m_rhs_variable(dof_family, solver_name + "RHSVariable")
  , m_solution_variable(dof_family, solver_name + "SolutionVariable")
  , m_dof_forced_info(dof_family, solver_name + "DoFForcedInfo")
  , m_dof_forced_value(dof_family, solver_name + "DoFForcedValue")
  , m_dof_elimination_info(dof_family, solver_name + "DoFEliminationInfo")
  , m_dof_elimination_value(dof_family, solver_name + "DoFEliminationValue")
  {}

  void clearValues() override
  {
    m_dof_forced_info.fill(false);
    m_dof_elimination_info.fill(ELIMINATE_NONE);
    m_dof_elimination_value.fill(0.0);
  }
  VariableDoFReal& solutionVariable() final { return m_solution_variable; }
  VariableDoFReal& rhsVariable() final { return m_rhs_variable; }
  VariableDoFBool& getForcedInfo() final { return m_dof_forced_info; }
  VariableDoFReal& getForcedValue() final { return m_dof_forced_value; }
  VariableDoFByte& getEliminationInfo() final { return m_dof_elimination_info; }
  VariableDoFReal& getEliminationValue() final { return m_dof_elimination_value; }
  void setRunner(const Runner& r) override { m_runner = r; }
  Runner runner() const override { return m_runner; }
  IItemFamily* dofFamily() const { return m_dof_family; }
  void setConstantMatrixSparsity(bool val) final { m_constant_matrix_sparsity = val; }
  void setConstantMatrixValues(bool val) final { m_constant_matrix_values = val; }
  bool isMatrixSparsityConstant() const final { return m_constant_matrix_sparsity; }
  bool isMatrixValuesConstant() const final { return m_constant_matrix_values; }

 private:
  IItemFamily* m_dof_family = nullptr;
  Runner m_runner;
  VariableDoFReal m_rhs_variable;
  VariableDoFReal m_solution_variable;
  VariableDoFBool m_dof_forced_info;
  VariableDoFReal m_dof_forced_value;
  VariableDoFByte m_dof_elimination_info;
  VariableDoFReal m_dof_elimination_value;
  bool m_constant_matrix_sparsity = false;
  bool m_constant_matrix_values = false;
};
} // namespace Arcane::FemUtils
