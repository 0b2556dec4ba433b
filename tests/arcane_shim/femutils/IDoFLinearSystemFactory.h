// Stand-in for femutils/IDoFLinearSystemFactory.h:34-44.
#pragma once
#include "FemUtilsGlobal.h"

namespace Arcane::FemUtils
{
class IDoFLinearSystemImpl;
class IDoFLinearSystemFactory
{
 public:
  virtual ~IDoFLinearSystemFactory() = default;
  virtual IDoFLinearSystemImpl* createInstance(ISubDomain* sd, IItemFamily* dof_family, const String& solver_name) = 0;
};
} // namespace Arcane::FemUtils
