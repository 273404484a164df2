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
#include <cstdint>
#include <cstdio>
#include <vector>

#include "morgana_gpu_epetra.hpp"
#include "morgana_gpu_tpetra.hpp"

template <typename T>
static void rd(FILE* f, T* p, size_t n)
{
  if (n && fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short read");
}

int main(int argc, char** argv)
{
  if (argc != 3) return 2;
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
    if (!T->isFillComplete() || T->Rows().size() != A->Rows().size()) return 9;
    for (const auto& row : A->Rows()) {
      auto it = T->Rows().find((long long)row.first);
      if (it == T->Rows().end() || it->second.size() != row.second.size()) return 9;
      for (size_t k = 0; k < row.second.size(); ++k)
        if ((long long)row.second[k].first != it->second[k].first || row.second[k].second != it->second[k].second)
          return 9;
    }

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
    std::vector<int32_t> rp(1, 0), col;
    std::vector<double> val;
    for (int64_t r = 0; r < ndof; ++r) {
      auto it = A->Rows().find((int)r);
      if (it != A->Rows().end())
        for (const auto& e : it->second) {
          col.push_back(e.first);
          val.push_back(e.second);
        }
      rp.push_back((int32_t)col.size());
    }
    const int64_t nz = (int64_t)col.size();
    fwrite(&ndof, sizeof(int64_t), 1, o);
    fwrite(&nz, sizeof(int64_t), 1, o);
    fwrite(rp.data(), sizeof(int32_t), rp.size(), o);
    fwrite(col.data(), sizeof(int32_t), col.size(), o);
    fwrite(val.data(), sizeof(double), val.size(), o);
    fwrite(Y[0], sizeof(double), ndof, o);
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
