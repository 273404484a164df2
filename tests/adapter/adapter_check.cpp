// Drives the Epetra and Tpetra adapters (include/morgana_gpu_epetra.hpp,
// include/morgana_gpu_tpetra.hpp) against the test doubles in mock_trilinos/:
// reads a mesh and coefficients written by the test, builds the operator through
// mg_epetra::buildEpetraCrs (and checks mg_tpetra::buildTpetraCrs inserts the
// same rows), applies it through mg_epetra::GpuCrsOperator, and writes what the
// Epetra side received.
//   adapter_check in.bin out.bin
// in.bin : int64 n_nodes, int64 n_elem, int64 order, double xyz[3 n_nodes],
//          int32 conn[4 n_elem], double kappa[n_elem], double x[ndof]
// out.bin: int64 ndof, int64 nnz, int32 rowptr[ndof+1], int32 col[nnz],
//          double val[nnz], double y[ndof]
// With a third argument "lagrange" it drives the boundary-multiplier pieces
// instead: B through mg_epetra::buildEpetraLagrange (and the same rows through
// mg_tpetra::buildTpetraLagrange), and the saddle matrix [K B^T; B 0] (K the
// kappa stiffness, card 4; B card 1) through mg_epetra::GpuSaddleOperator.
// in.bin : as above with x[ndof + n_multipliers]
// out.bin: int64 n_multipliers, int64 nnz_b, int32 rowptr[n_multipliers+1],
//          int32 col[nnz_b], double val[nnz_b], double y[ndof + n_multipliers]
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "morgana_gpu_epetra.hpp"
#include "morgana_gpu_tpetra.hpp"

template <typename T>
static void rd(FILE* f, T* p, size_t n)
{
  if (n && fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short read");
}

template <typename RowsA, typename RowsT>
static bool same_rows(const RowsA& a, const RowsT& t)
{
  if (a.size() != t.size()) return false;
  for (const auto& row : a) {
    auto it = t.find((long long)row.first);
    if (it == t.end() || it->second.size() != row.second.size()) return false;
    for (size_t k = 0; k < row.second.size(); ++k)
      if ((long long)row.second[k].first != it->second[k].first || row.second[k].second != it->second[k].second)
        return false;
  }
  return true;
}

template <typename Rows>
static void write_rows(FILE* o, const Rows& rows, int64_t nrows, const double* y, int64_t ny)
{
  std::vector<int32_t> rp(1, 0), col;
  std::vector<double> val;
  for (int64_t r = 0; r < nrows; ++r) {
    auto it = rows.find((int)r);
    if (it != rows.end())
      for (const auto& e : it->second) {
        col.push_back(e.first);
        val.push_back(e.second);
      }
    rp.push_back((int32_t)col.size());
  }
  const int64_t nz = (int64_t)col.size();
  fwrite(&nrows, sizeof(int64_t), 1, o);
  fwrite(&nz, sizeof(int64_t), 1, o);
  fwrite(rp.data(), sizeof(int32_t), rp.size(), o);
  fwrite(col.data(), sizeof(int32_t), col.size(), o);
  fwrite(val.data(), sizeof(double), val.size(), o);
  fwrite(y, sizeof(double), ny, o);
}

// the boundary-multiplier mode (see the head of this file)
static int run_lagrange(FILE* f, mg_plan* plan, int64_t ndof, int64_t nnz, int64_t ne,
                        const std::vector<double>& kappa, const char* out_path)
{
  mg_lagrange* lg = nullptr;
  mg_epetra::check(mg_lagrange_build(plan, 1, 0, nullptr, 0, &lg));
  mg_lagrange_info li{};
  mg_epetra::check(mg_lagrange_get_info(lg, &li));
  const int64_t n = ndof + li.n_multipliers;
  std::vector<double> x(n);
  rd(f, x.data(), x.size());
  fclose(f);

  Epetra_SerialComm comm;
  Teuchos::RCP<Epetra_FECrsMatrix> B = mg_epetra::buildEpetraLagrange(lg, MG_FACE_QUAD_1, comm);
  if (!B->Filled() || B->NumGlobalRange() != li.n_multipliers || B->NumGlobalDomain() != ndof) return 4;
  Teuchos::RCP<const Teuchos::Comm<int>> tcomm = Teuchos::rcp(new Teuchos::Comm<int>());
  Teuchos::RCP<mg_tpetra::crs_type> T = mg_tpetra::buildTpetraLagrange(lg, MG_FACE_QUAD_1, tcomm);
  if (!T->isFillComplete() || (int64_t)T->RangeSize() != li.n_multipliers || (int64_t)T->DomainSize() != ndof)
    return 9;
  if (!same_rows(B->Rows(), T->Rows())) return 9;

  double *dk = nullptr, *db = nullptr, *ds = nullptr, *dkappa = nullptr;
  if (cudaMalloc(&dk, sizeof(double) * (nnz > 0 ? nnz : 1)) != cudaSuccess ||
      cudaMalloc(&db, sizeof(double) * (li.nnz_b > 0 ? li.nnz_b : 1)) != cudaSuccess ||
      cudaMalloc(&ds, sizeof(double) * (li.nnz_saddle > 0 ? li.nnz_saddle : 1)) != cudaSuccess ||
      cudaMalloc(&dkappa, sizeof(double) * (ne > 0 ? ne : 1)) != cudaSuccess)
    return 5;
  cudaMemcpy(dkappa, kappa.data(), sizeof(double) * ne, cudaMemcpyHostToDevice);
  mg_epetra::check(mg_assemble(plan, MG_OP_STIFF_KAPPA, dkappa, 1.0, MG_QUAD_4, MG_F64, dk, nullptr));
  mg_epetra::check(mg_plan_status(plan));
  mg_epetra::check(mg_lagrange_assemble(lg, MG_FACE_QUAD_1, db, nullptr));
  mg_epetra::check(mg_saddle_assemble(lg, dk, db, nullptr, ds, nullptr));
  Epetra_Map map((int)n, 0, comm);
  Epetra_MultiVector X(map, 2), Y(map, 2);
  for (int64_t i = 0; i < n; ++i) {
    X[0][i] = x[i];
    X[1][i] = -x[i];
  }
  int rc;
  {
    mg_epetra::GpuSaddleOperator op(lg, ds, map);
    rc = op.Apply(X, Y);
  }
  if (rc != 0) return 6;
  for (int64_t i = 0; i < n; ++i)
    if (Y[1][i] != -Y[0][i]) return 7;

  FILE* o = fopen(out_path, "wb");
  if (!o) return 8;
  write_rows(o, B->Rows(), li.n_multipliers, Y[0], n);
  fclose(o);
  cudaFree(dk);
  cudaFree(db);
  cudaFree(ds);
  cudaFree(dkappa);
  mg_lagrange_destroy(lg);
  return 0;
}

int main(int argc, char** argv)
{
  if (argc != 3 && !(argc == 4 && std::string(argv[3]) == "lagrange")) return 2;
  try {
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 3;
    int64_t nn, ne, order;
    rd(f, &nn, 1);
    rd(f, &ne, 1);
    rd(f, &order, 1);
    std::vector<double> xyz(3 * nn), kappa(ne);
    std::vector<int32_t> conn(4 * ne);
    rd(f, xyz.data(), xyz.size());
    rd(f, conn.data(), conn.size());
    rd(f, kappa.data(), kappa.size());
    mg_mesh* mesh = nullptr;
    mg_plan* plan = nullptr;
    mg_epetra::check(mg_mesh_create(&mesh, nn, xyz.data(), ne, conn.data(), (int32_t)order, MG_EDGES_LEX));
    mg_epetra::check(mg_pattern_build(mesh, &plan));
    int64_t ndof = 0, nnz = 0;
    mg_epetra::check(mg_pattern_info(plan, &ndof, &nnz));
    if (argc == 4) {
      const int rc = run_lagrange(f, plan, ndof, nnz, ne, kappa, argv[2]);
      mg_plan_destroy(plan);
      mg_mesh_destroy(mesh);
      return rc;
    }
    std::vector<double> x(ndof);
    rd(f, x.data(), x.size());
    fclose(f);

    Epetra_SerialComm comm;
    Teuchos::RCP<Epetra_FECrsMatrix> A =
        mg_epetra::buildEpetraCrs(plan, MG_OP_STIFF_KAPPA, kappa.data(), 1.0, MG_QUAD_4, comm);
    if (!A->Filled()) return 4;

    // the Tpetra build inserts the same rows
    Teuchos::RCP<const Teuchos::Comm<int>> tcomm = Teuchos::rcp(new Teuchos::Comm<int>());
    Teuchos::RCP<mg_tpetra::crs_type> T =
        mg_tpetra::buildTpetraCrs(plan, MG_OP_STIFF_KAPPA, kappa.data(), 1.0, MG_QUAD_4, tcomm);
    if (!T->isFillComplete() || !same_rows(A->Rows(), T->Rows())) return 9;

    // the same operator on the device behind the Epetra_Operator seam
    double* dvals = nullptr;
    double* dkappa = nullptr;
    if (cudaMalloc(&dvals, sizeof(double) * (nnz > 0 ? nnz : 1)) != cudaSuccess) return 5;
    if (cudaMalloc(&dkappa, sizeof(double) * (ne > 0 ? ne : 1)) != cudaSuccess) return 5;
    cudaMemcpy(dkappa, kappa.data(), sizeof(double) * ne, cudaMemcpyHostToDevice);
    mg_epetra::check(mg_assemble(plan, MG_OP_STIFF_KAPPA, dkappa, 1.0, MG_QUAD_4, MG_F64, dvals, nullptr));
    mg_epetra::check(mg_plan_status(plan));
    Epetra_Map map((int)ndof, 0, comm);
    Epetra_MultiVector X(map, 2), Y(map, 2);
    for (int64_t i = 0; i < ndof; ++i) {
      X[0][i] = x[i];
      X[1][i] = 2.0 * x[i];
    }
    int rc;
    {
      mg_epetra::GpuCrsOperator op(plan, dvals, map);
      rc = op.Apply(X, Y);
    }
    if (rc != 0) return 6;
    for (int64_t i = 0; i < ndof; ++i)
      if (Y[1][i] != 2.0 * Y[0][i]) return 7;  // each column goes through the same SpMV

    FILE* o = fopen(argv[2], "wb");
    if (!o) return 8;
    write_rows(o, A->Rows(), ndof, Y[0], ndof);
    fclose(o);
    cudaFree(dvals);
    cudaFree(dkappa);
    mg_plan_destroy(plan);
    mg_mesh_destroy(mesh);
  } catch (const std::exception& e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
