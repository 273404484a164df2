/* Tpetra drop-in over the C ABI of libmorgana_gpu.so: header-only, compiled on
   the reference side where Trilinos exists.

   mg_tpetra::buildTpetraCrs gives the GPU-assembled operator as a filled
   Tpetra::CrsMatrix<> over a contiguous Tpetra::Map<> of the plan's dofs, what
   traitsMatrixBuilder<...>::buildTpetraCrs produces
   (src/morganaFiniteElements/traitsMatrixBuilder.hpp:546-623 in morganaPublic,
   with the default template arguments it uses, :79-85): one row per dof, index
   base 0, columns sorted, explicit zeros kept.  mg_tpetra::buildTpetraLagrange
   does the same for B of opLA3dA (rows over the boundary multipliers,
   fillComplete(field map, multiplier map)).  Errors from the C ABI are thrown
   as std::runtime_error with mg_last_error(). */
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "Teuchos_ArrayView.hpp"
#include "Teuchos_Comm.hpp"
#include "Teuchos_RCP.hpp"
#include "Tpetra_CrsMatrix.hpp"
#include "Tpetra_Map.hpp"
#include "morgana_gpu.h"

namespace mg_tpetra {

typedef Tpetra::Map<> map_type;
typedef Tpetra::CrsMatrix<> crs_type;

inline void check(mg_status s)
{
  if (s != MG_OK) throw std::runtime_error(std::string("libmorgana_gpu: ") + mg_last_error());
}

/* Operator `kind` (MG_OP_*) with per-element coefficient h_kappa (host,
   n_elements doubles, or NULL), constant c and quadrature card quad; MG_F64,
   repeated with MG_F64_NATIVE when the double-word range does not cover the
   element scales (MG_ERR_UNSUPPORTED). */
inline Teuchos::RCP<crs_type> buildTpetraCrs(mg_plan* plan, int32_t kind, const double* h_kappa, double c,
                                             int32_t quad, const Teuchos::RCP<const Teuchos::Comm<int>>& comm)
{
  typedef typename crs_type::global_ordinal_type GO;
  typedef typename crs_type::local_ordinal_type LO;
  typedef typename crs_type::scalar_type SC;
  int64_t ndof = 0, nnz = 0;
  check(mg_pattern_info(plan, &ndof, &nnz));
  std::vector<int32_t> rowptr(ndof + 1), colind(nnz);
  std::vector<double> values(nnz);
  check(mg_pattern_export(plan, rowptr.data(), colind.data()));
  mg_status st = mg_assemble_host(plan, kind, h_kappa, c, quad, MG_F64, values.data(), nullptr);
  if (st == MG_ERR_UNSUPPORTED)
    st = mg_assemble_host(plan, kind, h_kappa, c, quad, MG_F64_NATIVE, values.data(), nullptr);
  check(st);
  Teuchos::RCP<const map_type> rowMap = Teuchos::rcp(new map_type((Tpetra::global_size_t)ndof, (GO)0, comm));
  std::vector<size_t> perRow(ndof);
  for (int64_t r = 0; r < ndof; ++r) perRow[r] = (size_t)(rowptr[r + 1] - rowptr[r]);
  Teuchos::RCP<crs_type> matrix =
      Teuchos::rcp(new crs_type(rowMap, Teuchos::ArrayView<const size_t>(perRow.data(), (size_t)ndof)));
  std::vector<GO> cols;
  std::vector<SC> vals;
  for (int64_t r = 0; r < ndof; ++r) {
    const int32_t n = rowptr[r + 1] - rowptr[r];
    if (n == 0) continue;
    cols.assign(colind.begin() + rowptr[r], colind.begin() + rowptr[r + 1]);
    vals.assign(values.begin() + rowptr[r], values.begin() + rowptr[r + 1]);
    matrix->insertGlobalValues((GO)r, (LO)n, vals.data(), cols.data());
  }
  matrix->fillComplete();
  return matrix;
}

/* B (n_multipliers x ndof) of the multipliers lg with the face card quad (MG_FACE_QUAD_*). */
inline Teuchos::RCP<crs_type> buildTpetraLagrange(mg_lagrange* lg, int32_t quad,
                                                  const Teuchos::RCP<const Teuchos::Comm<int>>& comm)
{
  typedef typename crs_type::global_ordinal_type GO;
  typedef typename crs_type::local_ordinal_type LO;
  typedef typename crs_type::scalar_type SC;
  mg_lagrange_info li{};
  check(mg_lagrange_get_info(lg, &li));
  const int64_t nl = li.n_multipliers;
  std::vector<int32_t> rowptr(nl + 1), colind(li.nnz_b);
  std::vector<double> values(li.nnz_b);
  check(mg_lagrange_pattern(lg, rowptr.data(), colind.data(), nullptr, nullptr));
  check(mg_lagrange_assemble_host(lg, quad, values.data()));
  Teuchos::RCP<const map_type> rowMap = Teuchos::rcp(new map_type((Tpetra::global_size_t)nl, (GO)0, comm));
  Teuchos::RCP<const map_type> colMap = Teuchos::rcp(new map_type((Tpetra::global_size_t)li.ndof, (GO)0, comm));
  std::vector<size_t> perRow(nl + 1, 0);
  for (int64_t r = 0; r < nl; ++r) perRow[r] = (size_t)(rowptr[r + 1] - rowptr[r]);
  Teuchos::RCP<crs_type> matrix =
      Teuchos::rcp(new crs_type(rowMap, Teuchos::ArrayView<const size_t>(perRow.data(), (size_t)nl)));
  std::vector<GO> cols;
  std::vector<SC> vals;
  for (int64_t r = 0; r < nl; ++r) {
    const int32_t n = rowptr[r + 1] - rowptr[r];
    if (n == 0) continue;
    cols.assign(colind.begin() + rowptr[r], colind.begin() + rowptr[r + 1]);
    vals.assign(values.begin() + rowptr[r], values.begin() + rowptr[r + 1]);
    matrix->insertGlobalValues((GO)r, (LO)n, vals.data(), cols.data());
  }
  matrix->fillComplete(colMap, rowMap);
  return matrix;
}

}  // namespace mg_tpetra
