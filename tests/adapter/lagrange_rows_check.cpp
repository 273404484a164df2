// CPU check of the Trilinos pieces for the multipliers
// (mg_epetra::buildEpetraLagrange, mg_tpetra::buildTpetraLagrange) against the
// test doubles in mock_trilinos/: the multiplier space and patterns come from
// libmorgana_gpu.so's host-only calls; the values come from the definition of
// mg_lagrange_assemble_host below (this executable's own symbol takes
// precedence over the library's), known numbers that need no device.
//   lagrange_rows_check in.bin test_order
// in.bin: int64 n_nodes, int64 n_elem, int64 order, double xyz[3 n_nodes], int32 conn[4 n_elem]
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "morgana_gpu_epetra.hpp"
#include "morgana_gpu_tpetra.hpp"

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
    mg_epetra::check(mg_lagrange_build(plan, std::atoi(argv[2]), 0, nullptr, 0, &lg));
    mg_lagrange_info li{};
    mg_epetra::check(mg_lagrange_get_info(lg, &li));
    std::vector<int32_t> rp(li.n_multipliers + 1), ci(li.nnz_b);
    mg_epetra::check(mg_lagrange_pattern(lg, rp.data(), ci.data(), nullptr, nullptr));

    Epetra_SerialComm comm;
    Teuchos::RCP<Epetra_FECrsMatrix> B = mg_epetra::buildEpetraLagrange(lg, MG_FACE_QUAD_1, comm);
    if (!B->Filled() || B->NumGlobalRange() != li.n_multipliers || B->NumGlobalDomain() != li.ndof) return 4;
    Teuchos::RCP<const Teuchos::Comm<int>> tcomm = Teuchos::rcp(new Teuchos::Comm<int>());
    Teuchos::RCP<mg_tpetra::crs_type> T = mg_tpetra::buildTpetraLagrange(lg, MG_FACE_QUAD_1, tcomm);
    if (!T->isFillComplete() || (int64_t)T->RangeSize() != li.n_multipliers || (int64_t)T->DomainSize() != li.ndof)
      return 5;
    // every row as the pattern says, values in CSR order
    int64_t rows = 0;
    for (int64_t r = 0; r < li.n_multipliers; ++r) {
      const int32_t n = rp[r + 1] - rp[r];
      auto ie = B->Rows().find((int)r);
      auto it = T->Rows().find((long long)r);
      if (n == 0) {
        if (ie != B->Rows().end() || it != T->Rows().end()) return 6;
        continue;
      }
      if (ie == B->Rows().end() || it == T->Rows().end()) return 6;
      if ((int32_t)ie->second.size() != n || (int32_t)it->second.size() != n) return 7;
      for (int32_t k = 0; k < n; ++k) {
        const int32_t s = rp[r] + k;
        const double v = 0.25 * (double)s + 1.0;
        if (ie->second[k].first != ci[s] || ie->second[k].second != v) return 8;
        if (it->second[k].first != (long long)ci[s] || it->second[k].second != v) return 8;
      }
      ++rows;
    }
    if (rows != (int64_t)B->Rows().size()) return 9;
    mg_lagrange_destroy(lg);
    mg_plan_destroy(plan);
    mg_mesh_destroy(mesh);
  } catch (const std::exception& e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
