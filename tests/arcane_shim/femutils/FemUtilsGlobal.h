// Stand-in for femutils/FemUtilsGlobal.h: the CSRFormatView name and the
// elimination constants (femutils/FemUtilsGlobal.h:51-62).
#pragma once
#include <arcane/ArcaneShim.h>

namespace Arcane::FemUtils
{
class CsrFormatMatrixView;
using CSRFormatView = CsrFormatMatrixView;
static constexpr Byte ELIMINATE_NONE = 0;
static constexpr Byte ELIMINATE_ROW = 1;
static constexpr Byte ELIMINATE_ROW_COLUMN = 2;
} // namespace Arcane::FemUtils
