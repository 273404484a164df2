// Element matrices computed by the reference's own compiled code, for pinning
// the oracle (TEST INFRASTRUCTURE ONLY: built from the morganaPublic sources by
// oracle/ref/Makefile into oracle/_ref/, read by tests/golden/make_ref_elements.py
// to write golden fixtures; nothing in the product loads it).
//
// The pieces that carry the values are the reference's, compiled from its
// sources: the quadrature cards intStaticCard<linearTetra,STANDARD,P>
// (src/morganaIntegrator/intStaticCards.cpp:707-991), the P1/P2 basis polynomials
// through feStaticRealEval / feStaticRealDx,Dy,Dz
// (src/morganaFields/feStaticEvalIterators.hpp, feStaticLists.hpp:141-157,
// src/morganaPolynomial/polyCards.cpp), the Jacobian of the affine map
// geoMapInterface<linearTetra>::getGradient / getGradientDet
// (src/morganaGeometry/geoMapInterface.hpp:374-397) and tensor3d::computeInverse /
// getThirdInvariant (src/morganaDofs/tensor3d.cpp:400-484).  This file adds the
// glue the reference spreads over its class templates, in the same arithmetic
// order: fePr3d::globalGrad (src/morganaFields/fePr3d.hpp:418-442, 643-667), the
// integrands of opEL3dA / opEL3dF / opEL3dG / opEL3dM
// (src/morganaOperators/opEL3dA.hpp:129-165, opEL3dF.hpp:102-133,
// opEL3dG.hpp:83-108, opEL3dM.hpp:129-158) and the quadrature loop of
// integratorOEL3d_STD::integration (src/morganaIntegrator/integratorOEL3d_STD.hpp:106-137).
#include "typesInterface.hpp"
#include "geoMapInterface.hpp"
#include "intStaticCards.h"
#include "feStaticEvalIterators.hpp"

namespace {

enum { kStiffKappa = 0, kStiffConst = 1, kMass = 2, kMassCoeff = 3 };

// fePr3d::globalGrad: J from the element nodes, inverted in place, then the
// local gradients combined with the columns of J^-1
template <FELabel FE, UInt NB>
void global_grad(const sVect<point3d>& nodes, const point3d& Y, sVect<Real>& gx, sVect<Real>& gy, sVect<Real>& gz)
{
  geoMapInterface<linearTetra> geo;
  tensor3d T = geo.getGradient(nodes, Y);
  T.computeInverse();
  sVect<Real> lx(NB), ly(NB), lz(NB);
  feStaticRealDx<FE, NB>::eval(lx, Y);
  feStaticRealDy<FE, NB>::eval(ly, Y);
  feStaticRealDz<FE, NB>::eval(lz, Y);
  for (UInt i = 1; i <= NB; ++i) {
    gx(i) = lx(i) * T(1, 1) + ly(i) * T(2, 1) + lz(i) * T(3, 1);
    gy(i) = lx(i) * T(1, 2) + ly(i) * T(2, 2) + lz(i) * T(3, 2);
    gz(i) = lx(i) * T(1, 3) + ly(i) * T(2, 3) + lz(i) * T(3, 3);
  }
}

template <FELabel FE, UInt NB, UInt PREC>
void element(int op, const double* xyz, double kappa, double c, double* out)
{
  typedef intStaticCard<linearTetra, STANDARD, PREC> CARD;
  sVect<point3d> nodes(4);
  for (UInt s = 0; s < 4; ++s) nodes(s + 1) = point3d(xyz[3 * s], xyz[3 * s + 1], xyz[3 * s + 2]);
  geoMapInterface<linearTetra> geo;
  const UInt size = NB * NB;
  sVect<Real> mat(size), buf(size);
  for (UInt k = 1; k <= size; ++k) mat(k) = 0.0;
  for (UInt q = 1; q <= CARD::N; ++q) {
    const point3d Y = CARD::getYn(q);
    UInt tot = 1;
    if (op == kStiffKappa || op == kStiffConst) {
      // evalGrad_field and evalGrad_test: the same element, computed twice
      sVect<Real> fx(NB), fy(NB), fz(NB), tx(NB), ty(NB), tz(NB);
      global_grad<FE, NB>(nodes, Y, fx, fy, fz);
      global_grad<FE, NB>(nodes, Y, tx, ty, tz);
      const Real val = op == kStiffKappa ? kappa : c;
      for (UInt i = 1; i <= NB; ++i)
        for (UInt j = 1; j <= NB; ++j) {
          buf(tot) = (fx(i) * tx(j) + fy(i) * ty(j) + fz(i) * tz(j)) * val;
          ++tot;
        }
    } else {
      sVect<Real> vf(NB), vt(NB);
      feStaticRealEval<FE, NB>::eval(vf, Y);
      feStaticRealEval<FE, NB>::eval(vt, Y);
      for (UInt i = 1; i <= NB; ++i)
        for (UInt j = 1; j <= NB; ++j) {
          buf(tot) = op == kMass ? vf(i) * vt(j) : vf(i) * vt(j) * kappa;
          ++tot;
        }
    }
    const Real jac = geo.getGradientDet(nodes, Y);
    for (UInt k = 1; k <= size; ++k) mat(k) += buf(k) * jac * CARD::getWn(q);
  }
  for (UInt k = 0; k < size; ++k) out[k] = mat(k + 1);
}

template <FELabel FE, UInt NB>
int element_prec(int op, int prec, const double* xyz, double kappa, double c, double* out)
{
  switch (prec) {
    case 1: element<FE, NB, 1>(op, xyz, kappa, c, out); return 0;
    case 2: element<FE, NB, 2>(op, xyz, kappa, c, out); return 0;
    case 3: element<FE, NB, 3>(op, xyz, kappa, c, out); return 0;
    case 4: element<FE, NB, 4>(op, xyz, kappa, c, out); return 0;
  }
  return 1;
}

}  // namespace

extern "C" {

// Element matrix of one tet (xyz: 4 x 3 node coordinates in local order) for
// operator op (0 opEL3dA kappa, 1 opEL3dF c, 2 opEL3dG, 3 opEL3dM kappa), order
// 1 or 2, reference card precision 1..4; out[(i - 1) nb + (j - 1)] for field i,
// test j (the reference's column-major local layout).  Returns 0 on success.
int ref_local_matrix(int op, int order, int prec, const double* xyz, double kappa, double c, double* out)
{
  if (op < 0 || op > 3) return 1;
  if (order == 1) return element_prec<FE_P1_3d, 4>(op, prec, xyz, kappa, c, out);
  if (order == 2) return element_prec<FE_P2_3d, 10>(op, prec, xyz, kappa, c, out);
  return 1;
}

// The quadrature card itself (points and weights), for pinning the cards.
int ref_quad_rule(int prec, double* Y, double* W)
{
  auto fill = [&](auto card) {
    typedef decltype(card) CARD;
    for (UInt q = 1; q <= CARD::N; ++q) {
      const point3d p = CARD::getYn(q);
      Y[3 * (q - 1)] = p.getX();
      Y[3 * (q - 1) + 1] = p.getY();
      Y[3 * (q - 1) + 2] = p.getZ();
      W[q - 1] = CARD::getWn(q);
    }
    return (int)CARD::N;
  };
  switch (prec) {
    case 1: return fill(intStaticCard<linearTetra, STANDARD, 1>());
    case 2: return fill(intStaticCard<linearTetra, STANDARD, 2>());
    case 3: return fill(intStaticCard<linearTetra, STANDARD, 3>());
    case 4: return fill(intStaticCard<linearTetra, STANDARD, 4>());
  }
  return -1;
}

}  // extern "C"
