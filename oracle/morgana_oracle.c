/*
 * morgana_oracle.c -- CPU restatement of Morgana's finite-element operator path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke check and the cpu_baseline leg of the benchmark link it to compare the
 * CUDA path against, and to time the reference algorithm on host cores.  The
 * product library never links, loads or calls it.
 *
 * Every function follows a named piece of the reference (paths are relative to
 * the morganaPublic checkout) and keeps its arithmetic order where that order
 * fixes FP64 rounding:
 *
 *   quadrature tables    src/morganaIntegrator/intStaticCards.cpp:707-991
 *   P1/P2 monomials      src/morganaPolynomial/polyCards.cpp:232-285,
 *                        evaluated as src/morganaPolynomial/polyPow.hpp:97-158
 *   Jacobian             src/morganaGeometry/geoMapInterface.hpp:374-397
 *   det / inverse        src/morganaDofs/tensor3d.cpp:400-430, 478-484
 *   global gradients     src/morganaFields/fePr3d.hpp:418-442, 643-667
 *   integrand bodies     src/morganaOperators/opEL3dA.hpp:129-165 (kappa grad.grad)
 *                        src/morganaOperators/opEL3dF.hpp:102-133 (c grad.grad)
 *                        src/morganaOperators/opEL3dG.hpp:83-108  (u v)
 *                        src/morganaOperators/opEL3dM.hpp:129-158 (u v kappa)
 *                        src/morganaOperators/fnEL3dA.hpp:114-134, fnEL3dB.hpp:85-100
 *   quadrature loop      src/morganaIntegrator/integratorOEL3d_STD.hpp:106-137
 *                        src/morganaIntegrator/integratorFEL3d_STD.hpp:99-130
 *   edge enumeration     src/morganaGeometry/connect3d.hpp:417-491,
 *                        src/morganaGeometry/geoShapes.cpp:670-677
 *   edge numbering       src/morganaContainer/pVectGlobalManip.hpp:414-486 (pMapItem,
 *                        lexicographic on sorted node pairs, pGraphItem.cpp:236-260)
 *                        src/morganaContainer/pVectGlobalManip.hpp:498-578 with
 *                        traitsConnectOptimization.hpp:96-119 (pMapItemShare, 1 rank:
 *                        first appearance)
 *   dof numbering        src/morganaFields/dofMapStatic3d.hpp:420-560, 580-662
 *   CSR assembly         src/morganaFiniteElements/traitsMatrixBuilder.hpp:363-441
 *                        (column-major local block, row = test dof, duplicates summed
 *                        in insertion = element order, columns sorted, zeros kept)
 *   load vector          src/morganaFiniteElements/traitsVectorBuilder.hpp:214-274
 *   CG                   src/morganaTrilinos/belosBlockCG.hpp:46-82 (block size 1)
 *   boundary faces       src/morganaFiniteElements/localMatrixLA3d.hpp:292-322,
 *   (opLA3dA)            src/morganaIntegrator/integratorOLA3d_STD.hpp:102-124,
 *                        src/morganaOperators/opLA3dA.hpp:86-112,
 *                        src/morganaIntegrator/intStaticCards.cpp:176-300 (triangle cards)
 *
 * Build additions that have no reference counterpart (symmetric Dirichlet
 * elimination, adjoint gradient dJ/dkappa_e = -lambda_e^T Khat_e u_e) are marked
 * as such where they are defined.
 *
 * Indices are 0-based in every array this file takes or returns.
 * Compile with -ffp-contract=off so that x86 and Arm give the same bits.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_OK 0
#define OR_ERR_ARG 1
#define OR_ERR_MESH 4
#define OR_ERR_NOCONV 5

enum { OR_OP_STIFF_KAPPA = 0, OR_OP_STIFF_CONST = 1, OR_OP_MASS = 2, OR_OP_MASS_COEFF = 3 };
enum { OR_EDGES_LEX = 0, OR_EDGES_FIRST = 1 };

/* ------------------------------------------------------------------------- */
/* Quadrature on the reference tetrahedron (intStaticCards.cpp:707-991).      */
/* prec 1: 1 point, 2: 4 points, 3: 15 points, 4: 64 points (collapsed Gauss) */
/* ------------------------------------------------------------------------- */
int or_quad_rule(int prec, double *Y, double *W)
{
  if (prec == 1) {
    Y[0] = Y[1] = Y[2] = 1.0 / 4.0;
    W[0] = 1.0 / 6.0;
    return 1;
  }
  if (prec == 2) {
    const double a = (5.0 - sqrt(5.0)) / 20.0;
    const double b = (5.0 + 3 * sqrt(5.0)) / 20.0;
    const double P[4][3] = {{a, a, a}, {a, a, b}, {a, b, a}, {b, a, a}};
    for (int i = 0; i < 4; ++i) {
      Y[3 * i] = P[i][0]; Y[3 * i + 1] = P[i][1]; Y[3 * i + 2] = P[i][2];
      W[i] = 1.0 / 24.0;
    }
    return 4;
  }
  if (prec == 3) {
    const double r5 = 0.25;
    const double s5[2] = {0.09197107805272303, 0.3197936278296299};
    const double t5[2] = {0.7240867658418310, 0.04061911651111023};
    const double u5 = 0.05635083268962915;
    const double v5 = 0.4436491673103708;
    const double A5 = 0.01975308641975309;
    const double B5[2] = {0.01198951396316977, 0.01151136787104540};
    const double C5 = 0.008818342151675485;
    const double P[15][3] = {
        {r5, r5, r5},
        {s5[0], s5[0], s5[0]}, {t5[0], s5[0], s5[0]}, {s5[0], t5[0], s5[0]}, {s5[0], s5[0], t5[0]},
        {s5[1], s5[1], s5[1]}, {t5[1], s5[1], s5[1]}, {s5[1], t5[1], s5[1]}, {s5[1], s5[1], t5[1]},
        {u5, u5, v5}, {u5, v5, u5}, {v5, u5, u5}, {v5, v5, u5}, {v5, u5, v5}, {u5, v5, v5}};
    const double w[15] = {A5, B5[0], B5[0], B5[0], B5[0], B5[1], B5[1], B5[1], B5[1],
                          C5, C5, C5, C5, C5, C5};
    for (int i = 0; i < 15; ++i) {
      Y[3 * i] = P[i][0]; Y[3 * i + 1] = P[i][1]; Y[3 * i + 2] = P[i][2];
      W[i] = w[i];
    }
    return 15;
  }
  if (prec == 4) {
    const double t[4] = {0.0485005494, 0.2386007376, 0.5170472951, 0.7958514179};
    const double s[4] = {0.0571041961, 0.2768430136, 0.5835904324, 0.8602401357};
    const double r[4] = {0.0694318422, 0.3300094782, 0.6699905218, 0.9305681558};
    const double A[4] = {0.1739274226, 0.3260725774, 0.3260725774, 0.1739274226};
    const double B[4] = {0.1355069134, 0.2034645680, 0.1298475476, 0.0311809709};
    const double C[4] = {0.1108884156, 0.1434587898, 0.0686338872, 0.0103522407};
    /* point index = 16*c + 4*b + a  (r[c], s[b], t[a]); weight A[c'] B[b'] C[a'] in
       the reference's own (different) nesting: Wn[16*i + 4*j + k] = A[i]B[j]C[k]. */
    int n = 0;
    for (int c = 0; c < 4; ++c)
      for (int b = 0; b < 4; ++b)
        for (int a = 0; a < 4; ++a) {
          Y[3 * n] = t[a];
          Y[3 * n + 1] = s[b] * (1 - t[a]);
          Y[3 * n + 2] = r[c] * (1 - s[b]) * (1 - t[a]);
          ++n;
        }
    n = 0;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        for (int k = 0; k < 4; ++k) W[n++] = A[i] * B[j] * C[k];
    return 64;
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Reference basis (polyCards.cpp:232-285).  Each polynomial is a list of     */
/* monomials C x^px y^py z^pz summed left to right (polyEvalIter).            */
/* ------------------------------------------------------------------------- */
typedef struct { double C; int px, py, pz; } mono_t;

static const mono_t P1_A[4] = {{1, 0, 0, 0}, {-1, 1, 0, 0}, {-1, 0, 1, 0}, {-1, 0, 0, 1}};
static const mono_t P1_B[1] = {{1, 1, 0, 0}};
static const mono_t P1_C[1] = {{1, 0, 1, 0}};
static const mono_t P1_D[1] = {{1, 0, 0, 1}};

static const mono_t P2_A[10] = {{1, 0, 0, 0}, {-3, 1, 0, 0}, {-3, 0, 1, 0}, {-3, 0, 0, 1},
                                {2, 2, 0, 0}, {2, 0, 2, 0}, {2, 0, 0, 2},
                                {4, 1, 1, 0}, {4, 1, 0, 1}, {4, 0, 1, 1}};
static const mono_t P2_B[2] = {{2, 2, 0, 0}, {-1, 1, 0, 0}};
static const mono_t P2_C[2] = {{2, 0, 2, 0}, {-1, 0, 1, 0}};
static const mono_t P2_D[2] = {{2, 0, 0, 2}, {-1, 0, 0, 1}};
static const mono_t P2_E[4] = {{4, 1, 0, 0}, {-4, 2, 0, 0}, {-4, 1, 1, 0}, {-4, 1, 0, 1}};
static const mono_t P2_F[1] = {{4, 1, 1, 0}};
static const mono_t P2_G[4] = {{4, 0, 1, 0}, {-4, 1, 1, 0}, {-4, 0, 2, 0}, {-4, 0, 1, 1}};
static const mono_t P2_H[4] = {{4, 0, 0, 1}, {-4, 1, 0, 1}, {-4, 0, 1, 1}, {-4, 0, 0, 2}};
static const mono_t P2_I[1] = {{4, 1, 0, 1}};
static const mono_t P2_L[1] = {{4, 0, 1, 1}};

typedef struct { const mono_t *m; int n; } poly_t;
static const poly_t P1_LIST[4] = {{P1_A, 4}, {P1_B, 1}, {P1_C, 1}, {P1_D, 1}};
static const poly_t P2_LIST[10] = {{P2_A, 10}, {P2_B, 2}, {P2_C, 2}, {P2_D, 2}, {P2_E, 4},
                                   {P2_F, 1},  {P2_G, 4}, {P2_H, 4}, {P2_I, 1}, {P2_L, 1}};

/* polyPow<N>: ((1*x)*x)...; polySwitch<false> gives 0 for negative powers. */
static double ppow(double x, int n)
{
  if (n < 0) return 0.0;
  double r = 1.0;
  for (int i = 0; i < n; ++i) r = r * x;
  return r;
}

/* polyFactorial<D>(N) = N (N-1) ... (N-D+1) for D = 0 or 1 here. */
static double pfact(int d, int n) { return d == 0 ? 1.0 : (double)n; }

static double poly_eval(const poly_t *p, const double *Y)
{
  double v = 0.0;
  for (int s = 0; s < p->n; ++s) {
    const mono_t *m = &p->m[s];
    double t = m->C * ppow(Y[0], m->px) * ppow(Y[1], m->py) * ppow(Y[2], m->pz);
    v = (s == 0) ? t : v + t;
  }
  return v;
}

static double poly_der(const poly_t *p, int dx, int dy, int dz, const double *Y)
{
  double v = 0.0;
  for (int s = 0; s < p->n; ++s) {
    const mono_t *m = &p->m[s];
    double t = m->C * pfact(dx, m->px) * ppow(Y[0], m->px - dx) * pfact(dy, m->py) *
               ppow(Y[1], m->py - dy) * pfact(dz, m->pz) * ppow(Y[2], m->pz - dz);
    v = (s == 0) ? t : v + t;
  }
  return v;
}

static const poly_t *basis_list(int order) { return order == 1 ? P1_LIST : P2_LIST; }
static int nbasis(int order) { return order == 1 ? 4 : 10; }

void or_basis_eval(int order, const double *Y, double *val)
{
  const poly_t *L = basis_list(order);
  for (int i = 0; i < nbasis(order); ++i) val[i] = poly_eval(&L[i], Y);
}

void or_basis_grad(int order, const double *Y, double *gx, double *gy, double *gz)
{
  const poly_t *L = basis_list(order);
  for (int i = 0; i < nbasis(order); ++i) {
    gx[i] = poly_der(&L[i], 1, 0, 0, Y);
    gy[i] = poly_der(&L[i], 0, 1, 0, Y);
    gz[i] = poly_der(&L[i], 0, 0, 1, Y);
  }
}

/* ------------------------------------------------------------------------- */
/* Geometry (geoMapInterface.hpp:374-397, tensor3d.cpp:41-53,400-430,478-484) */
/* The linear-tet geometric map uses the P1 basis; column c of J is           */
/* sum_{s=4..1} x_s dphi_s/dxi_c accumulated as baseDerXIter does.            */
/* ------------------------------------------------------------------------- */
static void jacobian(const double *P /*4x3*/, const double *Y, double T[3][3])
{
  double gx[4], gy[4], gz[4];
  or_basis_grad(1, Y, gx, gy, gz);
  const double *g[3] = {gx, gy, gz};
  for (int c = 0; c < 3; ++c) {
    for (int r = 0; r < 3; ++r) {
      /* points(S)*d(S) + (points(S-1)*d(S-1) + ... (points(1)*d(1))) */
      double acc = P[0 * 3 + r] * g[c][0];
      for (int s = 1; s < 4; ++s) acc = P[s * 3 + r] * g[c][s] + acc;
      T[r][c] = acc;
    }
  }
}

static double third_invariant(double T[3][3])
{
  return T[0][0] * T[1][1] * T[2][2] - T[0][0] * T[1][2] * T[2][1] - T[1][0] * T[0][1] * T[2][2] +
         T[1][0] * T[0][2] * T[2][1] + T[2][0] * T[0][1] * T[1][2] - T[2][0] * T[0][2] * T[1][1];
}

static void compute_inverse(double T[3][3])
{
  double d = T[0][0] * T[1][1] * T[2][2] - T[0][0] * T[1][2] * T[2][1] - T[1][0] * T[0][1] * T[2][2] +
             T[1][0] * T[0][2] * T[2][1] + T[2][0] * T[0][1] * T[1][2] - T[2][0] * T[0][2] * T[1][1];
  double inv[3][3];
  inv[0][0] = (T[1][1] * T[2][2] - T[1][2] * T[2][1]) / d;
  inv[0][1] = -(T[0][1] * T[2][2] - T[0][2] * T[2][1]) / d;
  inv[0][2] = (T[0][1] * T[1][2] - T[0][2] * T[1][1]) / d;
  inv[1][0] = -(T[1][0] * T[2][2] - T[1][2] * T[2][0]) / d;
  inv[1][1] = (T[0][0] * T[2][2] - T[0][2] * T[2][0]) / d;
  inv[1][2] = -(T[0][0] * T[1][2] - T[0][2] * T[1][0]) / d;
  inv[2][0] = (T[1][0] * T[2][1] - T[1][1] * T[2][0]) / d;
  inv[2][1] = -(T[0][0] * T[2][1] - T[0][1] * T[2][0]) / d;
  inv[2][2] = (T[0][0] * T[1][1] - T[0][1] * T[1][0]) / d;
  memcpy(T, inv, sizeof(inv));
}

/* fePr3d::globalGrad: grad_i = locX*T(1,c) + locY*T(2,c) + locZ*T(3,c) with T = J^-1 */
static void global_grad(int order, const double *P, const double *Y, double *gx, double *gy,
                        double *gz)
{
  double T[3][3];
  jacobian(P, Y, T);
  compute_inverse(T);
  double lx[10], ly[10], lz[10];
  or_basis_grad(order, Y, lx, ly, lz);
  for (int i = 0; i < nbasis(order); ++i) {
    gx[i] = lx[i] * T[0][0] + ly[i] * T[1][0] + lz[i] * T[2][0];
    gy[i] = lx[i] * T[0][1] + ly[i] * T[1][1] + lz[i] * T[2][1];
    gz[i] = lx[i] * T[0][2] + ly[i] * T[1][2] + lz[i] * T[2][2];
  }
}

double or_element_det(const double *xyz, const int32_t *nodes4)
{
  double P[12];
  for (int s = 0; s < 4; ++s)
    for (int r = 0; r < 3; ++r) P[3 * s + r] = xyz[3 * (int64_t)nodes4[s] + r];
  const double Y[3] = {0.25, 0.25, 0.25};
  double T[3][3];
  jacobian(P, Y, T);
  return third_invariant(T);
}

/* ------------------------------------------------------------------------- */
/* Element matrix: integratorOEL3d_STD::integration with one of opEL3dA/F/G/M */
/* mat[i_field*nb + j_test], i.e. column-major with row = test (opColMajor).  */
/* ------------------------------------------------------------------------- */
int or_local_matrix(int op, int order, int quad, const double *xyz, const int32_t *nodes4,
                    double kappa, double c, double *mat)
{
  double Yq[64 * 3], Wq[64];
  int nq = or_quad_rule(quad, Yq, Wq);
  if (nq == 0) return OR_ERR_ARG;
  const int nb = nbasis(order);
  double P[12];
  for (int s = 0; s < 4; ++s)
    for (int r = 0; r < 3; ++r) P[3 * s + r] = xyz[3 * (int64_t)nodes4[s] + r];
  for (int k = 0; k < nb * nb; ++k) mat[k] = 0.0;
  double buf[100];
  for (int q = 0; q < nq; ++q) {
    const double *Y = &Yq[3 * q];
    if (op == OR_OP_STIFF_KAPPA || op == OR_OP_STIFF_CONST) {
      double fx[10], fy[10], fz[10], tx[10], ty[10], tz[10];
      global_grad(order, P, Y, fx, fy, fz); /* evalGrad_field */
      global_grad(order, P, Y, tx, ty, tz); /* evalGrad_test (second inverse) */
      /* P0 coefficient field: evalL = 0 + basis(=1)*dof */
      double val = (op == OR_OP_STIFF_KAPPA) ? 0.0 + 1.0 * kappa : c;
      int tot = 0;
      for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nb; ++j)
          buf[tot++] = (fx[i] * tx[j] + fy[i] * ty[j] + fz[i] * tz[j]) * val;
    } else {
      double fv[10], tv[10];
      or_basis_eval(order, Y, fv); /* globalEval == reference values */
      or_basis_eval(order, Y, tv);
      int tot = 0;
      if (op == OR_OP_MASS) {
        for (int i = 0; i < nb; ++i)
          for (int j = 0; j < nb; ++j) buf[tot++] = fv[i] * tv[j];
      } else if (op == OR_OP_MASS_COEFF) {
        double val = 0.0 + 1.0 * kappa;
        for (int i = 0; i < nb; ++i)
          for (int j = 0; j < nb; ++j) buf[tot++] = fv[i] * tv[j] * val;
      } else {
        return OR_ERR_ARG;
      }
    }
    double T[3][3];
    jacobian(P, Y, T);
    double jac = third_invariant(T); /* signed, no abs */
    for (int k = 0; k < nb * nb; ++k) mat[k] += buf[k] * jac * Wq[q];
  }
  return OR_OK;
}

/* Load vector of one element: integratorFEL3d_STD with fnEL3dA (field != NULL:
   the coefficient is the nodal field of the same P1/P2 space, evaluated as
   feStaticField3d::evalL) or fnEL3dB (field == NULL). */
int or_local_vector(int order, int quad, const double *xyz, const int32_t *nodes4,
                    const double *field_local, double *vec)
{
  double Yq[64 * 3], Wq[64];
  int nq = or_quad_rule(quad, Yq, Wq);
  if (nq == 0) return OR_ERR_ARG;
  const int nb = nbasis(order);
  double P[12];
  for (int s = 0; s < 4; ++s)
    for (int r = 0; r < 3; ++r) P[3 * s + r] = xyz[3 * (int64_t)nodes4[s] + r];
  for (int k = 0; k < nb; ++k) vec[k] = 0.0;
  for (int q = 0; q < nq; ++q) {
    const double *Y = &Yq[3 * q];
    double tv[10], buf[10];
    or_basis_eval(order, Y, tv);
    if (field_local) {
      double val = 0.0;
      for (int i = 0; i < nb; ++i) val += tv[i] * field_local[i];
      for (int j = 0; j < nb; ++j) buf[j] = tv[j] * val;
    } else {
      for (int j = 0; j < nb; ++j) buf[j] = tv[j];
    }
    double T[3][3];
    jacobian(P, Y, T);
    double jac = third_invariant(T);
    for (int j = 0; j < nb; ++j) vec[j] += buf[j] * jac * Wq[q];
  }
  return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* Mesh checks (meshDoctor3d.hpp:195-227): detJ > 0 at the reference vertices */
/* ------------------------------------------------------------------------- */
int or_check_jacobian(int64_t n_elem, const double *xyz, const int32_t *conn, double *min_det,
                      int64_t *first_bad)
{
  double mn = INFINITY;
  *first_bad = -1;
  for (int64_t e = 0; e < n_elem; ++e) {
    double P[12];
    for (int s = 0; s < 4; ++s)
      for (int r = 0; r < 3; ++r) P[3 * s + r] = xyz[3 * (int64_t)conn[4 * e + s] + r];
    static const double V[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int v = 0; v < 4; ++v) {
      double T[3][3];
      jacobian(P, V[v], T);
      double d = third_invariant(T);
      if (d < mn) mn = d;
      if (!(d > 0.0) && *first_bad < 0) *first_bad = e;
    }
  }
  *min_det = mn;
  return *first_bad < 0 ? OR_OK : OR_ERR_MESH;
}

/* ------------------------------------------------------------------------- */
/* Edges (connect3d.hpp:417-491).  Local edge j of a tet joins local vertices  */
/* edgeToPoint(j,.) = (1,2),(2,3),(3,1),(1,4),(2,4),(3,4).  Edge lids follow   */
/* first appearance in the element x local-edge loop; the global numbering is  */
/* either lexicographic on the sorted node pair (pMapItem) or the lid order    */
/* itself (pMapItemShare on one rank, every edge local).                       */
/* elem_edge[E*6] receives 0-based global edge numbers, edge_nodes[nE*2] the   */
/* two node ids of each global edge in its first-seen local orientation.       */
/* ------------------------------------------------------------------------- */
static const int EDGE_TO_POINT[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};

typedef struct { int64_t key; int64_t idx; } kv_t;

static int cmp_kv(const void *a, const void *b)
{
  const kv_t *x = (const kv_t *)a, *y = (const kv_t *)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

int or_build_edges(int64_t n_nodes, int64_t n_elem, const int32_t *conn, int rule,
                   int32_t *elem_edge, int32_t *edge_nodes, int64_t *n_edges_out)
{
  int64_t m = 6 * n_elem;
  kv_t *kv = (kv_t *)malloc(sizeof(kv_t) * (size_t)(m > 0 ? m : 1));
  if (!kv) return OR_ERR_ARG;
  for (int64_t e = 0; e < n_elem; ++e)
    for (int j = 0; j < 6; ++j) {
      int64_t a = conn[4 * e + EDGE_TO_POINT[j][0]], b = conn[4 * e + EDGE_TO_POINT[j][1]];
      int64_t lo = a < b ? a : b, hi = a < b ? b : a;
      kv[6 * e + j].key = lo * n_nodes + hi;
      kv[6 * e + j].idx = 6 * e + j;
    }
  qsort(kv, (size_t)m, sizeof(kv_t), cmp_kv);
  /* lex rank of each unique edge, and the first occurrence (smallest idx). */
  int64_t nE = 0;
  int64_t *first = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m > 0 ? m : 1));
  int32_t *lex_of = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m > 0 ? m : 1));
  for (int64_t k = 0; k < m; ++k) {
    if (k == 0 || kv[k].key != kv[k - 1].key) {
      first[nE] = kv[k].idx; /* sorted by idx inside equal keys */
      ++nE;
    }
    lex_of[kv[k].idx] = (int32_t)(nE - 1);
  }
  /* first-appearance rank of each unique edge */
  int32_t *fa_of_lex = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nE > 0 ? nE : 1));
  {
    kv_t *fk = (kv_t *)malloc(sizeof(kv_t) * (size_t)(nE > 0 ? nE : 1));
    for (int64_t u = 0; u < nE; ++u) { fk[u].key = first[u]; fk[u].idx = u; }
    qsort(fk, (size_t)nE, sizeof(kv_t), cmp_kv);
    for (int64_t r = 0; r < nE; ++r) fa_of_lex[fk[r].idx] = (int32_t)r;
    free(fk);
  }
  for (int64_t k = 0; k < m; ++k) {
    int32_t lx = lex_of[k];
    elem_edge[k] = (rule == OR_EDGES_LEX) ? lx : fa_of_lex[lx];
  }
  for (int64_t u = 0; u < nE; ++u) {
    int64_t idx = first[u];
    int64_t e = idx / 6;
    int j = (int)(idx % 6);
    int32_t g = (rule == OR_EDGES_LEX) ? (int32_t)u : fa_of_lex[u];
    edge_nodes[2 * g] = conn[4 * e + EDGE_TO_POINT[j][0]];
    edge_nodes[2 * g + 1] = conn[4 * e + EDGE_TO_POINT[j][1]];
  }
  *n_edges_out = nE;
  free(kv); free(first); free(lex_of); free(fa_of_lex);
  return OR_OK;
}

/* dofMapStatic3d (allMode, vectMajor, Real dofs): vertex dof = node gid,
   edge dof = numVerticesG + edge gid; list gid - 1 gives the 0-based index. */
void or_elem_dofs(int order, int64_t n_nodes, int64_t n_elem, const int32_t *conn,
                  const int32_t *elem_edge, int32_t *dofs)
{
  const int nb = nbasis(order);
  for (int64_t e = 0; e < n_elem; ++e) {
    for (int v = 0; v < 4; ++v) dofs[nb * e + v] = conn[4 * e + v];
    if (order == 2)
      for (int j = 0; j < 6; ++j) dofs[nb * e + 4 + j] = (int32_t)(n_nodes + elem_edge[6 * e + j]);
  }
}

/* ------------------------------------------------------------------------- */
/* CSR pattern: union of element couplings, explicit zeros kept, columns      */
/* sorted (what Epetra GlobalAssemble leaves behind).                         */
/* ------------------------------------------------------------------------- */
static int cmp_i32(const void *a, const void *b)
{
  int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

int or_pattern(int order, int64_t ndof, int64_t n_elem, const int32_t *dofs, int32_t *rowptr,
               int32_t *colind, int64_t cap, int64_t *nnz_out)
{
  const int nb = nbasis(order);
  /* rows -> incident (element, local) via counting sort */
  int64_t *cnt = (int64_t *)calloc((size_t)ndof + 1, sizeof(int64_t));
  for (int64_t k = 0; k < n_elem * nb; ++k) cnt[dofs[k] + 1]++;
  for (int64_t r = 0; r < ndof; ++r) cnt[r + 1] += cnt[r];
  int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ndof + 1));
  memcpy(pos, cnt, sizeof(int64_t) * (size_t)(ndof + 1));
  int64_t *inc = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n_elem * nb > 0 ? n_elem * nb : 1));
  for (int64_t k = 0; k < n_elem * nb; ++k) inc[pos[dofs[k]]++] = k / nb;
  /* the row buffer holds the couplings of the row with the most incidences */
  int64_t max_inc = 1;
  for (int64_t r = 0; r < ndof; ++r)
    if (cnt[r + 1] - cnt[r] > max_inc) max_inc = cnt[r + 1] - cnt[r];
  int32_t *tmp = (int32_t *)malloc(sizeof(int32_t) * (size_t)(max_inc * nb));
  int64_t nnz = 0;
  rowptr[0] = 0;
  for (int64_t r = 0; r < ndof; ++r) {
    int64_t n = 0;
    for (int64_t t = cnt[r]; t < cnt[r + 1]; ++t) {
      int64_t e = inc[t];
      for (int i = 0; i < nb; ++i) tmp[n++] = dofs[nb * e + i];
    }
    qsort(tmp, (size_t)n, sizeof(int32_t), cmp_i32);
    for (int64_t t = 0; t < n; ++t) {
      if (t > 0 && tmp[t] == tmp[t - 1]) continue;
      if (nnz >= cap) { free(cnt); free(pos); free(inc); free(tmp); return OR_ERR_ARG; }
      colind[nnz++] = tmp[t];
    }
    rowptr[r + 1] = (int32_t)nnz;
  }
  *nnz_out = nnz;
  free(cnt); free(pos); free(inc); free(tmp);
  return OR_OK;
}

static int64_t find_slot(const int32_t *rowptr, const int32_t *colind, int32_t row, int32_t col)
{
  int64_t lo = rowptr[row], hi = rowptr[row + 1] - 1;
  while (lo <= hi) {
    int64_t mid = (lo + hi) / 2;
    if (colind[mid] == col) return mid;
    if (colind[mid] < col) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

/* buildEpetraCrs: element loop, InsertGlobalValues(COLUMN_MAJOR), GlobalAssemble.
   Each (row, col) sums its contributions in element order, starting from 0. */
int or_assemble_values(int op, int order, int quad, const double *xyz, int64_t n_elem,
                       const int32_t *conn, const int32_t *dofs, const double *coeff, double c,
                       const int32_t *rowptr, const int32_t *colind, int64_t ndof, double *values)
{
  const int nb = nbasis(order);
  memset(values, 0, sizeof(double) * (size_t)rowptr[ndof]);
  double mat[100];
  for (int64_t e = 0; e < n_elem; ++e) {
    double kappa = coeff ? coeff[e] : 1.0;
    int rc = or_local_matrix(op, order, quad, xyz, &conn[4 * e], kappa, c, mat);
    if (rc) return rc;
    for (int i = 0; i < nb; ++i)      /* field (column) */
      for (int j = 0; j < nb; ++j) {  /* test (row) */
        int64_t s = find_slot(rowptr, colind, dofs[nb * e + j], dofs[nb * e + i]);
        if (s < 0) return OR_ERR_ARG;
        values[s] += mat[i * nb + j];
      }
  }
  return OR_OK;
}

/* vectorBuilder::buildEpetraVector: SumIntoGlobalValues in element order.
   field (ndof nodal values) may be NULL (fnEL3dB); elem_scale (E) is a build
   addition that multiplies each element's vector (NULL = 1). */
int or_assemble_rhs(int order, int quad, const double *xyz, int64_t n_elem, const int32_t *conn,
                    const int32_t *dofs, const double *field, const double *elem_scale, int64_t ndof,
                    double *b)
{
  const int nb = nbasis(order);
  memset(b, 0, sizeof(double) * (size_t)ndof);
  double vec[10], fl[10];
  for (int64_t e = 0; e < n_elem; ++e) {
    if (field)
      for (int i = 0; i < nb; ++i) fl[i] = field[dofs[nb * e + i]];
    int rc = or_local_vector(order, quad, xyz, &conn[4 * e], field ? fl : NULL, vec);
    if (rc) return rc;
    double s = elem_scale ? elem_scale[e] : 1.0;
    for (int j = 0; j < nb; ++j) b[dofs[nb * e + j]] += elem_scale ? vec[j] * s : vec[j];
  }
  return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* Build addition (no reference counterpart; the reference imposes Dirichlet  */
/* data through Lagrange multipliers): symmetric elimination of masked dofs.  */
/* Row and column of a masked dof are zeroed, its diagonal set to 1, rhs 0.   */
/* ------------------------------------------------------------------------- */
void or_apply_dirichlet(int64_t ndof, const int32_t *rowptr, const int32_t *colind,
                        const uint8_t *mask, double *values, double *b)
{
  for (int64_t r = 0; r < ndof; ++r) {
    for (int64_t s = rowptr[r]; s < rowptr[r + 1]; ++s) {
      int32_t c = colind[s];
      if (mask[r]) values[s] = (c == r) ? 1.0 : 0.0;
      else if (mask[c]) values[s] = 0.0;
    }
    if (b && mask[r]) b[r] = 0.0;
  }
}

/* ------------------------------------------------------------------------- */
/* CSR SpMV and conjugate gradients (the operator Belos consumes).            */
/* ------------------------------------------------------------------------- */
void or_spmv(int64_t ndof, const int32_t *rowptr, const int32_t *colind, const double *values,
             const double *x, double *y)
{
  for (int64_t r = 0; r < ndof; ++r) {
    double acc = 0.0;
    for (int64_t s = rowptr[r]; s < rowptr[r + 1]; ++s) acc += values[s] * x[colind[s]];
    y[r] = acc;
  }
}

static double dot(int64_t n, const double *a, const double *b)
{
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* Preconditioned CG (precond 0 = none, 1 = Jacobi); stops when
   ||r||_2 <= rtol ||b||_2.  Returns iterations through *iters and the final
   relative residual through *relres. */
int or_cg(int64_t ndof, const int32_t *rowptr, const int32_t *colind, const double *values,
          const double *b, double *x, double rtol, int maxit, int precond, int *iters,
          double *relres)
{
  double *r = (double *)malloc(sizeof(double) * (size_t)ndof);
  double *z = (double *)malloc(sizeof(double) * (size_t)ndof);
  double *p = (double *)malloc(sizeof(double) * (size_t)ndof);
  double *q = (double *)malloc(sizeof(double) * (size_t)ndof);
  double *dinv = (double *)malloc(sizeof(double) * (size_t)ndof);
  for (int64_t i = 0; i < ndof; ++i) {
    double d = 1.0;
    if (precond == 1) {
      d = 0.0;
      for (int64_t s = rowptr[i]; s < rowptr[i + 1]; ++s)
        if (colind[s] == i) d = values[s];
    }
    dinv[i] = (d != 0.0) ? 1.0 / d : 1.0;
  }
  or_spmv(ndof, rowptr, colind, values, x, q);
  for (int64_t i = 0; i < ndof; ++i) { r[i] = b[i] - q[i]; z[i] = dinv[i] * r[i]; p[i] = z[i]; }
  double bn = sqrt(dot(ndof, b, b));
  if (bn == 0.0) bn = 1.0;
  double rz = dot(ndof, r, z);
  double rn = sqrt(dot(ndof, r, r));
  int it = 0;
  while (rn > rtol * bn && it < maxit) {
    or_spmv(ndof, rowptr, colind, values, p, q);
    double alpha = rz / dot(ndof, p, q);
    for (int64_t i = 0; i < ndof; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
    for (int64_t i = 0; i < ndof; ++i) z[i] = dinv[i] * r[i];
    double rz_new = dot(ndof, r, z);
    double beta = rz_new / rz;
    rz = rz_new;
    for (int64_t i = 0; i < ndof; ++i) p[i] = z[i] + beta * p[i];
    rn = sqrt(dot(ndof, r, r));
    ++it;
  }
  *iters = it;
  *relres = rn / bn;
  free(r); free(z); free(p); free(q); free(dinv);
  return rn <= rtol * bn ? OR_OK : OR_ERR_NOCONV;
}

/* ------------------------------------------------------------------------- */
/* Build addition: adjoint gradient of J(kappa) with respect to a P0 kappa.   */
/* dJ/dkappa_e = -lambda_e^T Khat_e u_e, Khat_e the opEL3dA element matrix at */
/* kappa_e = 1 (K_e is linear in kappa_e).                                    */
/* ------------------------------------------------------------------------- */
int or_adjoint_grad(int order, int quad, const double *xyz, int64_t n_elem, const int32_t *conn,
                    const int32_t *dofs, const double *u, const double *lambda, double *grad)
{
  const int nb = nbasis(order);
  double mat[100];
  for (int64_t e = 0; e < n_elem; ++e) {
    int rc = or_local_matrix(OR_OP_STIFF_KAPPA, order, quad, xyz, &conn[4 * e], 1.0, 0.0, mat);
    if (rc) return rc;
    double s = 0.0;
    for (int i = 0; i < nb; ++i)
      for (int j = 0; j < nb; ++j)
        s += lambda[dofs[nb * e + j]] * mat[i * nb + j] * u[dofs[nb * e + i]];
    grad[e] = -s;
  }
  return OR_OK;
}

/* ------------------------------------------------------------------------- */
/* Boundary-face Lagrange operator opLA3dA: field = the tet's P1/P2 basis,    */
/* test = the P1 basis of the boundary triangle (fePr2d<1>).                  */
/* ------------------------------------------------------------------------- */

/* Triangle cards (intStaticCards.cpp:176-300): precision 1 = centroid,
   2 = edge midpoints, 3 = the 4-point rule with one negative weight,
   4 = the 6-point rule.  Y holds (x, y) pairs. */
int or_tri_rule(int prec, double *Y, double *W)
{
  if (prec == 1) {
    Y[0] = 1.0 / 3.0; Y[1] = 1.0 / 3.0;
    W[0] = 0.5;
    return 1;
  }
  if (prec == 2) {
    const double P[3][2] = {{0.5, 0.0}, {0.0, 0.5}, {0.5, 0.5}};
    for (int i = 0; i < 3; ++i) { Y[2 * i] = P[i][0]; Y[2 * i + 1] = P[i][1]; W[i] = 1.0 / 6.0; }
    return 3;
  }
  if (prec == 3) {
    const double a = 3.0 / 5.0, b = 1.0 / 5.0, c = 1.0 / 3.0;
    const double P[4][2] = {{a, b}, {b, a}, {b, b}, {c, c}};
    const double w[4] = {25.0 / 96.0, 25.0 / 96.0, 25.0 / 96.0, -9.0 / 32.0};
    for (int i = 0; i < 4; ++i) { Y[2 * i] = P[i][0]; Y[2 * i + 1] = P[i][1]; W[i] = w[i]; }
    return 4;
  }
  if (prec == 4) {
    const double x1 = 0.091576213509770743, x2 = 0.44594849091596488;
    const double w1 = 0.054975871827660933, w2 = 0.11169079483900573;
    const double P[6][2] = {{x1, x1}, {x1, 1 - 2 * x1}, {1 - 2 * x1, x1},
                            {x2, x2}, {x2, 1 - 2 * x2}, {1 - 2 * x2, x2}};
    const double w[6] = {w1, w1, w1, w2, w2, w2};
    for (int i = 0; i < 6; ++i) { Y[2 * i] = P[i][0]; Y[2 * i + 1] = P[i][1]; W[i] = w[i]; }
    return 6;
  }
  return 0;
}

/* Local faces of linearTetra (geoShapes.cpp:681-688), 0-based vertex indices. */
static const int FACE_PTS[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {0, 3, 2}};
static const double REF_TET[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

/* Local matrix of opLA3dA on local face lf (0..3) of a tet: the quadrature
   loop of integratorOLA3d_STD.hpp:102-124 around the integrand of
   opLA3dA.hpp:86-112,
     mat[a * nb + i] = sum_q (phi_i(Yv) psi_a(Ys)) |Vx ^ Vy| w_q,
   i over the tet's nb basis functions and a over the test basis of the
   boundary triangle: test_order 1 (fePr2d<1>) the face's points in face order,
   test_order 0 (fePr2d<0>) the one constant psi = 1, test_order 2 (fePr2d<2>)
   the three vertex functions l_a (2 l_a - 1) then the edge functions
   4 l_p l_q of the face's edges (0,1), (1,2), (2,0).
   Vx, Vy: derivatives of the linear map of the reference triangle onto the
   face (geoMapInterface.hpp:25-90, point 3 first).  Yv: the same map onto the
   reference tet's face (supportLagrange3d mapVolumeY).  Ys: the point in the
   boundary triangle's own coordinates (mapSurfaceY, through mapGlobalToLocal);
   the boundary triangle has the face's vertices, so psi_a(Ys) is the face
   barycentric a of the point, which this restatement uses directly (the two
   agree to rounding). */
int or_face_matrix(int order, int test_order, int prec, const double *xyz, const int32_t *nodes4, int lf,
                   double *mat)
{
  if (lf < 0 || lf > 3 || test_order < 0 || test_order > 2) return OR_ERR_ARG;
  const int nt = test_order == 2 ? 6 : (test_order == 1 ? 3 : 1);
  double Y[12], W[6];
  const int nq = or_tri_rule(prec, Y, W);
  if (nq == 0) return OR_ERR_ARG;
  const int nb = nbasis(order);
  double P[3][3];
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < 3; ++k) P[a][k] = xyz[3 * nodes4[FACE_PTS[lf][a]] + k];
  double Vx[3], Vy[3], N[3];
  for (int k = 0; k < 3; ++k) {
    Vx[k] = P[2][k] * 0.0 + (P[1][k] * 1.0 + P[0][k] * -1.0);
    Vy[k] = P[2][k] * 1.0 + (P[1][k] * 0.0 + P[0][k] * -1.0);
  }
  N[0] = Vx[1] * Vy[2] - Vx[2] * Vy[1];
  N[1] = Vx[2] * Vy[0] - Vx[0] * Vy[2];
  N[2] = Vx[0] * Vy[1] - Vx[1] * Vy[0];
  const double area2 = sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
  for (int k = 0; k < nt * nb; ++k) mat[k] = 0.0;
  for (int q = 0; q < nq; ++q) {
    const double x = Y[2 * q], y = Y[2 * q + 1];
    const double lam[3] = {1.0 - x - y, x, y};
    const double one[1] = {1.0};
    const double p2[6] = {lam[0] * (2 * lam[0] - 1), lam[1] * (2 * lam[1] - 1), lam[2] * (2 * lam[2] - 1),
                          4 * lam[0] * lam[1], 4 * lam[1] * lam[2], 4 * lam[2] * lam[0]};
    const double *psi = test_order == 2 ? p2 : (test_order == 1 ? lam : one);
    double Yv[3], phi[10];
    for (int k = 0; k < 3; ++k)
      Yv[k] = REF_TET[FACE_PTS[lf][2]][k] * lam[2] +
              (REF_TET[FACE_PTS[lf][1]][k] * lam[1] + REF_TET[FACE_PTS[lf][0]][k] * lam[0]);
    or_basis_eval(order, Yv, phi);
    for (int a = 0; a < nt; ++a)
      for (int i = 0; i < nb; ++i) mat[a * nb + i] += phi[i] * psi[a] * area2 * W[q];
  }
  return OR_OK;
}

/* or_face_matrix over a list of faces (face_elem[f], face_local[f]). */
int or_face_matrices(int order, int test_order, int prec, const double *xyz, int64_t n_faces,
                     const int32_t *conn, const int32_t *face_elem, const int32_t *face_local, double *out)
{
  const int nb = nbasis(order), nt = test_order == 2 ? 6 : (test_order == 1 ? 3 : 1);
  for (int64_t f = 0; f < n_faces; ++f) {
    int rc = or_face_matrix(order, test_order, prec, xyz, &conn[4 * (int64_t)face_elem[f]], face_local[f],
                            out + nt * nb * f);
    if (rc) return rc;
  }
  return OR_OK;
}
