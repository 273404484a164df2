/* Epetra drop-in pieces over the C ABI of libmorgana_gpu.so: header-only,
   compiled on the reference side where Trilinos exists.

   - mg_epetra::buildEpetraCrs: the GPU-assembled operator as a new
     Epetra_FECrsMatrix (pattern + values of one bilinear form), what
     traitsMatrixBuilder<...>::buildEpetraCrs produces
     (src/morganaFiniteElements/traitsMatrixBuilder.hpp:363-441 in morganaPublic):
     one row per dof, index base 0, columns sorted, explicit zeros kept.
   - mg_epetra::GpuCrsOperator: an Epetra_Operator whose Apply is mg_spmv on
     device-resident CSR values, the seam through which Belos / ML consume an
     operator (the Epetra_Operator interface of
     src/morganaTrilinos/epetraOperatorSum.h:32-77).

   - mg_epetra::buildEpetraLagrange: B of opLA3dA (boundary multipliers x field)
     as the Epetra_FECrsMatrix the same builder produces for localMatrixLA3d
     (src/morganaFiniteElements/localMatrixLA3d.hpp:292-322): rows over the
     multipliers, GlobalAssemble(field map, multiplier map); it feeds the
     reference's epetraSaddleAssembler::setSymmMatrix unchanged.
   - mg_epetra::GpuSaddleOperator: an Epetra_Operator whose Apply is
     mg_saddle_spmv on device-resident saddle values [K B^T; B 0].

   The builders take an mg_plan built by mg_pattern_build (or
   mg_pattern_build_device), or an mg_lagrange built over one; errors from the C
   ABI are thrown as std::runtime_error with mg_last_error(). */
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "Epetra_Comm.h"
#include "Epetra_FECrsMatrix.h"
#include "Epetra_Map.h"
#include "Epetra_MultiVector.h"
#include "Epetra_Operator.h"
#include "Teuchos_RCP.hpp"
#include "morgana_gpu.h"

namespace mg_epetra {

inline void check(mg_status s)
{
  if (s != MG_OK) throw std::runtime_error(std::string("libmorgana_gpu: ") + mg_last_error());
}

/* Pattern and values of operator `kind` (MG_OP_*) with per-element coefficient
   h_kappa (host, n_elements doubles; NULL for the constant / plain operators),
   constant c and quadrature card quad, as a filled Epetra_FECrsMatrix over a
   contiguous row map of the plan's dofs.  MG_F64 first; when its double-word
   range does not cover the element scales (MG_ERR_UNSUPPORTED) the call is
   repeated with MG_F64_NATIVE. */
inline Teuchos::RCP<Epetra_FECrsMatrix> buildEpetraCrs(mg_plan* plan, int32_t kind, const double* h_kappa, double c,
                                                       int32_t quad, const Epetra_Comm& comm)
{
  int64_t ndof = 0, nnz = 0;
  check(mg_pattern_info(plan, &ndof, &nnz));
  std::vector<int32_t> rowptr(ndof + 1), colind(nnz);
  std::vector<double> values(nnz);
  check(mg_pattern_export(plan, rowptr.data(), colind.data()));
  mg_status st = mg_assemble_host(plan, kind, h_kappa, c, quad, MG_F64, values.data(), nullptr);
  if (st == MG_ERR_UNSUPPORTED)
    st = mg_assemble_host(plan, kind, h_kappa, c, quad, MG_F64_NATIVE, values.data(), nullptr);
  check(st);
  Epetra_Map rowMap((int)ndof, 0, comm);
  std::vector<int> perRow(ndof);
  for (int64_t r = 0; r < ndof; ++r) perRow[r] = rowptr[r + 1] - rowptr[r];
  Teuchos::RCP<Epetra_FECrsMatrix> matrix =
      Teuchos::rcp(new Epetra_FECrsMatrix(Copy, rowMap, perRow.data()));
  for (int64_t r = 0; r < ndof; ++r)
    if (perRow[r] > 0) matrix->InsertGlobalValues((int)r, perRow[r], &values[rowptr[r]], &colind[rowptr[r]]);
  matrix->GlobalAssemble();
  return matrix;
}

/* y = A x for Belos / ML: the CSR values stay on the device (d_values, nnz
   doubles, e.g. from mg_assemble), vectors are copied in and out per column. */
class GpuCrsOperator : public Epetra_Operator
{
 public:
  GpuCrsOperator(mg_plan* plan, const double* d_values, const Epetra_Map& map)
      : plan_(plan), vals_(d_values), map_(map)
  {
    int64_t nnz = 0;
    check(mg_pattern_info(plan, &n_, &nnz));
    if (cudaMalloc(&dx_, sizeof(double) * (n_ > 0 ? n_ : 1)) != cudaSuccess ||
        cudaMalloc(&dy_, sizeof(double) * (n_ > 0 ? n_ : 1)) != cudaSuccess)
      throw std::runtime_error("GpuCrsOperator: device allocation failed");
  }
  ~GpuCrsOperator() override
  {
    cudaFree(dx_);
    cudaFree(dy_);
  }
  GpuCrsOperator(const GpuCrsOperator&) = delete;
  GpuCrsOperator& operator=(const GpuCrsOperator&) = delete;

  int Apply(const Epetra_MultiVector& X, Epetra_MultiVector& Y) const override
  {
    if (X.NumVectors() != Y.NumVectors() || X.MyLength() != (int)n_ || Y.MyLength() != (int)n_) return -1;
    const size_t bytes = sizeof(double) * (size_t)n_;
    for (int v = 0; v < X.NumVectors(); ++v) {
      if (cudaMemcpy(dx_, X[v], bytes, cudaMemcpyHostToDevice) != cudaSuccess) return -2;
      if (mg_spmv(plan_, MG_F64, vals_, dx_, dy_, nullptr) != MG_OK) return -3;
      if (cudaMemcpy(Y[v], dy_, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return -2;
    }
    return 0;
  }
  int ApplyInverse(const Epetra_MultiVector&, Epetra_MultiVector&) const override { return -1; }
  int SetUseTranspose(bool use) override { return use ? -1 : 0; }  // symmetric operators only
  double NormInf() const override { return 0.0; }
  const char* Label() const override { return "mg_epetra::GpuCrsOperator"; }
  bool UseTranspose() const override { return false; }
  bool HasNormInf() const override { return false; }
  const Epetra_Comm& Comm() const override { return map_.Comm(); }
  const Epetra_Map& OperatorDomainMap() const override { return map_; }
  const Epetra_Map& OperatorRangeMap() const override { return map_; }

 private:
  mg_plan* plan_;
  const double* vals_;
  const Epetra_Map& map_;
  int64_t n_ = 0;
  double* dx_ = nullptr;
  double* dy_ = nullptr;
};

/* B (n_multipliers x ndof) of the multipliers lg with the face card quad
   (MG_FACE_QUAD_*; the reference's default intDefault precision is card 1). */
inline Teuchos::RCP<Epetra_FECrsMatrix> buildEpetraLagrange(mg_lagrange* lg, int32_t quad, const Epetra_Comm& comm)
{
  mg_lagrange_info li{};
  check(mg_lagrange_get_info(lg, &li));
  std::vector<int32_t> rowptr(li.n_multipliers + 1), colind(li.nnz_b);
  std::vector<double> values(li.nnz_b);
  check(mg_lagrange_pattern(lg, rowptr.data(), colind.data(), nullptr, nullptr));
  check(mg_lagrange_assemble_host(lg, quad, values.data()));
  Epetra_Map rowMap((int)li.n_multipliers, 0, comm);
  Epetra_Map colMap((int)li.ndof, 0, comm);
  std::vector<int> perRow(li.n_multipliers + 1, 0);
  for (int64_t r = 0; r < li.n_multipliers; ++r) perRow[r] = rowptr[r + 1] - rowptr[r];
  Teuchos::RCP<Epetra_FECrsMatrix> matrix = Teuchos::rcp(new Epetra_FECrsMatrix(Copy, rowMap, perRow.data()));
  for (int64_t r = 0; r < li.n_multipliers; ++r)
    if (perRow[r] > 0) matrix->InsertGlobalValues((int)r, perRow[r], &values[rowptr[r]], &colind[rowptr[r]]);
  matrix->GlobalAssemble(colMap, rowMap);
  return matrix;
}

/* y = S x on the saddle matrix (values on the device, e.g. from
   mg_saddle_assemble); map: ndof + n_multipliers elements, field first. */
class GpuSaddleOperator : public Epetra_Operator
{
 public:
  GpuSaddleOperator(mg_lagrange* lg, const double* d_values, const Epetra_Map& map)
      : lg_(lg), vals_(d_values), map_(map)
  {
    mg_lagrange_info li{};
    check(mg_lagrange_get_info(lg, &li));
    n_ = li.ndof + li.n_multipliers;
    if (cudaMalloc(&dx_, sizeof(double) * (n_ > 0 ? n_ : 1)) != cudaSuccess ||
        cudaMalloc(&dy_, sizeof(double) * (n_ > 0 ? n_ : 1)) != cudaSuccess)
      throw std::runtime_error("GpuSaddleOperator: device allocation failed");
  }
  ~GpuSaddleOperator() override
  {
    cudaFree(dx_);
    cudaFree(dy_);
  }
  GpuSaddleOperator(const GpuSaddleOperator&) = delete;
  GpuSaddleOperator& operator=(const GpuSaddleOperator&) = delete;

  int Apply(const Epetra_MultiVector& X, Epetra_MultiVector& Y) const override
  {
    if (X.NumVectors() != Y.NumVectors() || X.MyLength() != (int)n_ || Y.MyLength() != (int)n_) return -1;
    const size_t bytes = sizeof(double) * (size_t)n_;
    for (int v = 0; v < X.NumVectors(); ++v) {
      if (cudaMemcpy(dx_, X[v], bytes, cudaMemcpyHostToDevice) != cudaSuccess) return -2;
      if (mg_saddle_spmv(lg_, vals_, dx_, dy_, nullptr) != MG_OK) return -3;
      if (cudaMemcpy(Y[v], dy_, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return -2;
    }
    return 0;
  }
  int ApplyInverse(const Epetra_MultiVector&, Epetra_MultiVector&) const override { return -1; }
  int SetUseTranspose(bool use) override { return use ? -1 : 0; }  // the saddle matrix is symmetric
  double NormInf() const override { return 0.0; }
  const char* Label() const override { return "mg_epetra::GpuSaddleOperator"; }
  bool UseTranspose() const override { return false; }
  bool HasNormInf() const override { return false; }
  const Epetra_Comm& Comm() const override { return map_.Comm(); }
  const Epetra_Map& OperatorDomainMap() const override { return map_; }
  const Epetra_Map& OperatorRangeMap() const override { return map_; }

 private:
  mg_lagrange* lg_;
  const double* vals_;
  const Epetra_Map& map_;
  int64_t n_ = 0;
  double* dx_ = nullptr;
  double* dy_ = nullptr;
};

}  // namespace mg_epetra
