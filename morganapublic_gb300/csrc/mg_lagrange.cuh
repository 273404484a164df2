// Boundary-face Lagrange operator opLA3dA: the per-face arithmetic, written once
// for the kernel (mg_lagrange.cu) and for a host build of the same code that
// the tests compare with the oracle on the CPU.  Plain FP64 arithmetic and
// integer tables only (no CUDA types, no static arrays).
//
// Face f is local face lf of tet e.  Its local matrix, rows = the test basis of
// the boundary triangle (P1: the face's three vertices in face order; P0: the
// constant 1; P2: the vertex functions l_a (2 l_a - 1), then 4 l_p l_q on the
// face's edges (0,1), (1,2), (2,0)), columns = the tet's nb field basis
// functions, is
//   mat[a * nb + i] = sum_q w_q |Vx ^ Vy| psi_a(q) phi_i(q)
// (integratorOLA3d_STD.hpp:102-124 around opLA3dA.hpp:86-112).  On the face the
// tet's barycentric coordinates are the face's own (lambda_a at vertex
// face_vertex(lf, a), zero at the opposite vertex), so phi_i is evaluated from
// them directly: P1 phi_v = L_v; P2 phi_v = L_v (2 L_v - 1), phi_{4+j} = 4 L_p L_q
// for local edge j = (p, q).
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define MG_HD __host__ __device__
#else
#define MG_HD
#endif

namespace mg {

// Local faces of linearTetra (geoShapes.cpp:681-688), 0-based: face lf has
// vertices {0,2,1}, {0,1,3}, {1,2,3}, {0,3,2}; 4 bits per vertex, 12 per face.
constexpr unsigned long long kFaceVerts = 0x120ull | (0x310ull << 12) | (0x321ull << 24) | (0x230ull << 36);
MG_HD inline int face_vertex(int lf, int a) { return (int)((kFaceVerts >> (12 * lf + 4 * a)) & 0xfull); }

// Local edges of linearTetra (geoShapes.cpp:670-677), 0-based: (0,1) (1,2)
// (2,0) (0,3) (1,3) (2,3); 4 bits per vertex, 8 per edge.
constexpr unsigned long long kEdgeVerts =
    0x10ull | (0x21ull << 8) | (0x02ull << 16) | (0x30ull << 24) | (0x31ull << 32) | (0x32ull << 40);
MG_HD inline int edge_vertex(int j, int s) { return (int)((kEdgeVerts >> (8 * j + 4 * s)) & 0xfull); }

// Triangle quadrature, points (x, y) on the reference triangle (0,0) (1,0)
// (0,1) and weights summing to 1/2.  Cards by point count: 1 (centroid), 3
// (edge midpoints), 4 (Strang-Fix, one negative weight), 6 (degree 4), the
// reference's STANDARD cards of precision 1..4 (intStaticCards.cpp:176-300).
struct FaceRule {
  int nq;
  double x[6], y[6], w[6];
};

inline bool face_rule(int quad, FaceRule* r)
{
  auto set = [r](int q, double x, double y, double w) { r->x[q] = x; r->y[q] = y; r->w[q] = w; };
  if (quad == 1) {
    r->nq = 1;
    set(0, 1.0 / 3.0, 1.0 / 3.0, 0.5);
  } else if (quad == 3) {
    r->nq = 3;
    set(0, 0.5, 0.0, 1.0 / 6.0);
    set(1, 0.0, 0.5, 1.0 / 6.0);
    set(2, 0.5, 0.5, 1.0 / 6.0);
  } else if (quad == 4) {
    r->nq = 4;
    const double a = 3.0 / 5.0, b = 1.0 / 5.0, w = 25.0 / 96.0;
    set(0, a, b, w);
    set(1, b, a, w);
    set(2, b, b, w);
    set(3, 1.0 / 3.0, 1.0 / 3.0, -9.0 / 32.0);
  } else if (quad == 6) {
    r->nq = 6;
    const double x1 = 0.091576213509770743, x2 = 0.44594849091596488;
    const double w1 = 0.054975871827660933, w2 = 0.11169079483900573;
    set(0, x1, x1, w1);
    set(1, x1, 1 - 2 * x1, w1);
    set(2, 1 - 2 * x1, x1, w1);
    set(3, x2, x2, w2);
    set(4, x2, 1 - 2 * x2, w2);
    set(5, 1 - 2 * x2, x2, w2);
  } else {
    return false;
  }
  return true;
}

// Local matrix of local face lf; P[a] = coordinates of face vertex a (face
// order), mat = NT x NB, row-major (test basis, field basis); NT = 3 (P1 test),
// 1 (P0 test) or 6 (P2 test).
template <int NB, int NT>
MG_HD inline void face_matrix(const double P[3][3], int lf, const FaceRule& r, double* mat)
{
  double vx[3], vy[3];
  for (int k = 0; k < 3; ++k) {
    vx[k] = P[1][k] - P[0][k];
    vy[k] = P[2][k] - P[0][k];
  }
  const double n0 = vx[1] * vy[2] - vx[2] * vy[1];
  const double n1 = vx[2] * vy[0] - vx[0] * vy[2];
  const double n2 = vx[0] * vy[1] - vx[1] * vy[0];
  const double area2 = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
  static_assert(NT == 1 || NT == 3 || NT == 6, "P0, P1 or P2 test basis");
  for (int k = 0; k < NT * NB; ++k) mat[k] = 0.0;
  for (int q = 0; q < r.nq; ++q) {
    const double lam[3] = {1.0 - r.x[q] - r.y[q], r.x[q], r.y[q]};
    double L[4] = {0.0, 0.0, 0.0, 0.0};
    for (int a = 0; a < 3; ++a) L[face_vertex(lf, a)] = lam[a];
    double phi[NB];
    if constexpr (NB == 4) {
      for (int v = 0; v < 4; ++v) phi[v] = L[v];
    } else {
      for (int v = 0; v < 4; ++v) phi[v] = L[v] * (2.0 * L[v] - 1.0);
      for (int j = 0; j < 6; ++j) phi[4 + j] = 4.0 * L[edge_vertex(j, 0)] * L[edge_vertex(j, 1)];
    }
    double psi[NT];
    if constexpr (NT == 1) {
      psi[0] = 1.0;
    } else if constexpr (NT == 3) {
      for (int a = 0; a < 3; ++a) psi[a] = lam[a];
    } else {
      for (int a = 0; a < 3; ++a) psi[a] = lam[a] * (2.0 * lam[a] - 1.0);
      for (int j = 0; j < 3; ++j) psi[3 + j] = 4.0 * lam[j] * lam[j == 2 ? 0 : j + 1];
    }
    const double s = area2 * r.w[q];
    for (int a = 0; a < NT; ++a) {
      const double c = psi[a] * s;
      for (int i = 0; i < NB; ++i) mat[a * NB + i] += phi[i] * c;
    }
  }
}

}  // namespace mg
