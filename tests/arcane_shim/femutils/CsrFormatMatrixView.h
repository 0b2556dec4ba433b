// Stand-in for femutils/CsrFormatMatrixView.h:135-210: the view's public
// accessors with the reference's layout -- rows() holds nbRow() row starts
// and no trailing entry, the last row ends at nbColumn(), unused slots of
// columns() hold -1.  The reference builds it only through CsrFormat (a
// friend); the shim's make() plays that role for the tests.
#pragma once
#include "FemUtilsGlobal.h"

namespace Arcane::FemUtils
{
class CsrFormatMatrixView
{
 public:
  CsrFormatMatrixView() = default;
  static CsrFormatMatrixView make(SmallSpan<const Int32> rows, SmallSpan<const Int32> rows_nb_column,
                                  SmallSpan<const Int32> columns, SmallSpan<Real> values)
  {
    CsrFormatMatrixView v;
    v.m_matrix_rows = rows;
    v.m_matrix_rows_nb_column = rows_nb_column;
    v.m_matrix_columns = columns;
    v.m_values = values;
    return v;
  }
  Span<const Int32> rows() const { return m_matrix_rows; }
  Span<const Int32> columns() const { return m_matrix_columns; }
  Span<Real> values() const { return m_values; }
  Int32 nbRow() const { return (Int32)m_matrix_rows.size(); }
  Int32 nbColumn() const { return (Int32)m_matrix_columns.size(); }
  Int32 nbValue() const { return (Int32)m_values.size(); }
  Int32 nbColumnForRow(Int32 row) const { return m_matrix_rows_nb_column[row]; }

 private:
  SmallSpan<const Int32> m_matrix_rows;
  SmallSpan<const Int32> m_matrix_rows_nb_column;
  SmallSpan<const Int32> m_matrix_columns;
  SmallSpan<Real> m_values;
};
} // namespace Arcane::FemUtils
