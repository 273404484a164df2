// CPU check of the Trilinos builders (mg_epetra::buildEpetraCrs,
// mg_tpetra::buildTpetraCrs, and for the multipliers buildEpetraLagrange,
// buildTpetraLagrange) against the test doubles in mock_trilinos/: meshes,
// plans, multiplier spaces and patterns come from libmorgana_gpu.so's
// host-only calls; the values come from the definitions of mg_assemble_host
// and mg_lagrange_assemble_host below (this executable's own symbols take
// precedence over the library's), known numbers that need no device.
//   rows_check in.bin test_order
// in.bin: int64 n_nodes, int64 n_elem, int64 order, double xyz[3 n_nodes], int32 conn[4 n_elem]
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "morgana_gpu_epetra.hpp"
#include "morgana_gpu_tpetra.hpp"

extern "C" mg_status mg_assemble_host(mg_plan* plan, int32_t, const double*, double, int32_t, int32_t,
                                      void* h_values, void*)
{
  int64_t ndof = 0, nnz = 0;
  mg_pattern_info(plan, &ndof, &nnz);
  for (int64_t k = 0; k < nnz; ++k) static_cast<double*>(h_values)[k] = 0.5 * (double)k - 3.0;
  return MG_OK;
}

extern "C" mg_status mg_lagrange_assemble_host(mg_lagrange* lg, int32_t, double* h_b_values)
{
  mg_lagrange_info li{};
  mg_lagrange_get_info(lg, &li);
  for (int64_t k = 0; k < li.nnz_b; ++k) h_b_values[k] = 0.25 * (double)k + 1.0;
  return MG_OK;
}

template <typename T>
static void rd(FILE* f, T* p, size_t n)
{
  if (n && fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short read");
}

// Epetra rows `re` and Tpetra rows `rt` both equal the CSR (rp, ci) with value(s)
template <typename RowsE, typename RowsT, typename V>
static bool rows_match(const RowsE& re, const RowsT& rt, const std::vector<int32_t>& rp,
                       const std::vector<int32_t>& ci, V value)
{
  int64_t rows = 0;
  for (int64_t r = 0; r + 1 < (int64_t)rp.size(); ++r) {
    const int32_t n = rp[r + 1] - rp[r];
    auto ie = re.find((int)r);
    auto it = rt.find((long long)r);
    if (n == 0) {
      if (ie != re.end() || it != rt.end()) return false;
      continue;
    }
    if (ie == re.end() || it == rt.end()) return false;
    if ((int32_t)ie->second.size() != n || (int32_t)it->second.size() != n) return false;
    for (int32_t k = 0; k < n; ++k) {
      const int32_t s = rp[r] + k;
      if (ie->second[k].first != ci[s] || ie->second[k].second != value(s)) return false;
      if (it->second[k].first != (long long)ci[s] || it->second[k].second != value(s)) return false;
    }
    ++rows;
  }
  return rows == (int64_t)re.size() && rows == (int64_t)rt.size();
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
    std::vector<double> xyz(3 * nn);
    std::vector<int32_t> conn(4 * ne);
    rd(f, xyz.data(), xyz.size());
    rd(f, conn.data(), conn.size());
    fclose(f);
    mg_mesh* mesh = nullptr;
    mg_plan* plan = nullptr;
    mg_lagrange* lg = nullptr;
    mg_epetra::check(mg_mesh_create(&mesh, nn, xyz.data(), ne, conn.data(), (int32_t)order, MG_EDGES_LEX));
    mg_epetra::check(mg_pattern_build(mesh, &plan));
    Epetra_SerialComm comm;
    Teuchos::RCP<const Teuchos::Comm<int>> tcomm = Teuchos::rcp(new Teuchos::Comm<int>());
    // K through buildEpetraCrs / buildTpetraCrs
    {
      int64_t ndof = 0, nnz = 0;
      mg_epetra::check(mg_pattern_info(plan, &ndof, &nnz));
      std::vector<int32_t> rp(ndof + 1), ci(nnz);
      mg_epetra::check(mg_pattern_export(plan, rp.data(), ci.data()));
      Teuchos::RCP<Epetra_FECrsMatrix> A = mg_epetra::buildEpetraCrs(plan, MG_OP_STIFF_CONST, nullptr, 1.0, MG_QUAD_4, comm);
      Teuchos::RCP<mg_tpetra::crs_type> AT =
          mg_tpetra::buildTpetraCrs(plan, MG_OP_STIFF_CONST, nullptr, 1.0, MG_QUAD_4, tcomm);
      if (!A->Filled() || !AT->isFillComplete()) return 10;
      if (!rows_match(A->Rows(), AT->Rows(), rp, ci, [](int32_t s) { return 0.5 * (double)s - 3.0; })) return 11;
    }
    mg_epetra::check(mg_lagrange_build(plan, std::atoi(argv[2]), 0, nullptr, 0, &lg));
    mg_lagrange_info li{};
    mg_epetra::check(mg_lagrange_get_info(lg, &li));
    std::vector<int32_t> rp(li.n_multipliers + 1), ci(li.nnz_b);
    mg_epetra::check(mg_lagrange_pattern(lg, rp.data(), ci.data(), nullptr, nullptr));

    Teuchos::RCP<Epetra_FECrsMatrix> B = mg_epetra::buildEpetraLagrange(lg, MG_FACE_QUAD_1, comm);
    if (!B->Filled() || B->NumGlobalRange() != li.n_multipliers || B->NumGlobalDomain() != li.ndof) return 4;
    Teuchos::RCP<mg_tpetra::crs_type> T = mg_tpetra::buildTpetraLagrange(lg, MG_FACE_QUAD_1, tcomm);
    if (!T->isFillComplete() || (int64_t)T->RangeSize() != li.n_multipliers || (int64_t)T->DomainSize() != li.ndof)
      return 5;
    if (!rows_match(B->Rows(), T->Rows(), rp, ci, [](int32_t s) { return 0.25 * (double)s + 1.0; })) return 6;
    mg_lagrange_destroy(lg);
    mg_plan_destroy(plan);
    mg_mesh_destroy(mesh);
  } catch (const std::exception& e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
