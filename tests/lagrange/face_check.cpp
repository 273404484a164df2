// Test harness: the per-face arithmetic of the boundary-face kernel
// (mg_lagrange.cuh, the body k_face_matrix runs per thread) built for the host,
// so the CPU tests can compare it with the oracle without a GPU.  Not part of
// the library.
#include <cstdint>

#include "mg_lagrange.cuh"

extern "C" int face_check_matrices(int order, int test_order, int quad, const double* xyz, int64_t n_faces,
                                   const int32_t* conn, const int32_t* face_elem, const int32_t* face_local,
                                   double* out)
{
  mg::FaceRule rule{};
  if (!mg::face_rule(quad, &rule)) return 1;
  const int nb = order == 1 ? 4 : 10, nt = test_order == 2 ? 6 : (test_order == 1 ? 3 : 1);
  for (int64_t f = 0; f < n_faces; ++f) {
    const int32_t* c = conn + 4 * (int64_t)face_elem[f];
    const int lf = face_local[f];
    double P[3][3];
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 3; ++k) P[a][k] = xyz[3 * (int64_t)c[mg::face_vertex(lf, a)] + k];
    double* o = out + f * nt * nb;
    if (nb == 4 && nt == 3) mg::face_matrix<4, 3>(P, lf, rule, o);
    else if (nb == 4 && nt == 1) mg::face_matrix<4, 1>(P, lf, rule, o);
    else if (nb == 4) mg::face_matrix<4, 6>(P, lf, rule, o);
    else if (nt == 3) mg::face_matrix<10, 3>(P, lf, rule, o);
    else if (nt == 1) mg::face_matrix<10, 1>(P, lf, rule, o);
    else mg::face_matrix<10, 6>(P, lf, rule, o);
  }
  return 0;
}
