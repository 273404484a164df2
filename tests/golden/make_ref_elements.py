"""Generates tests/golden/ref_elements.npz: element matrices and quadrature cards
computed by the reference's own code, compiled from a morganaPublic checkout by
oracle/ref/Makefile (the reference's quadrature cards, P1/P2 basis polynomials,
affine-map Jacobian, tensor3d inverse and determinant, driven through the
opEL3dA/F/G/M integrands and the integratorOEL3d_STD quadrature loop; see
oracle/ref/ref_element.cpp).

Contents:
  card{p}_Y, card{p}_W   intStaticCard<linearTetra,STANDARD,p>, p = 1..4
  xyz                    (16, 4, 3) tets: the 8 tets of the reference's test mesh
                         mignon3dC.msh (tests/golden/mignon3dC.json, local node
                         order as in the file), then 8 tets of a Kuhn cube
                         (2^3 cells, jitter 0.3h, seed 5)
  kappa                  (16,) the P0 coefficient: 12 on the mignon3dC tets (the
                         coefficient of the reference's integratorOEL3d_STDTest1),
                         lognormal (sigma 1, seed 6) on the others
  c                      the constant of opEL3dF (1: its matrix is the kappa-free
                         stiffness K^ of the adjoint gradient)
  m_{op}_{order}_{p}     (16, nb, nb) element matrices, [field i, test j], for op in
                         stiff_kappa / stiff_const / mass / mass_coeff, order 1 / 2

Run: python tests/golden/make_ref_elements.py <morganaPublic checkout>
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OPS = ["stiff_kappa", "stiff_const", "mass", "mass_coeff"]


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_ref_elements.py <morganaPublic checkout>")
    ref = os.path.abspath(sys.argv[1])
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={ref}"], check=True)
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libmorgana_ref.so"))
    L.ref_local_matrix.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_void_p]
    L.ref_quad_rule.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    sys.path.insert(0, ROOT)
    from morganapublic_gb300 import meshgen

    out = {}
    for p in (1, 2, 3, 4):
        Y, W = np.zeros((64, 3)), np.zeros(64)
        n = L.ref_quad_rule(p, Y.ctypes.data, W.ctypes.data)
        out[f"card{p}_Y"], out[f"card{p}_W"] = Y[:n].copy(), W[:n].copy()
    mig = json.load(open(os.path.join(HERE, "mignon3dC.json")))
    nodes = np.array(mig["nodes"], dtype=np.float64)
    tets = np.array(mig["tets_1based"], dtype=np.int64) - 1
    cube = meshgen.kuhn_cube(2, jitter=0.3, seed=5)
    xyz = np.concatenate([nodes[tets], cube.xyz[cube.conn[:8]]]).astype(np.float64)
    kappa = np.concatenate([np.full(len(tets), 12.0), meshgen.lognormal(8, 1.0, 6)])
    c = 1.0
    out["xyz"], out["kappa"], out["c"] = xyz, kappa, np.array(c)
    for op_id, op in enumerate(OPS):
        for order, nb in ((1, 4), (2, 10)):
            for p in (1, 2, 3, 4):
                mats = np.zeros((len(xyz), nb, nb))
                for t in range(len(xyz)):
                    buf = np.zeros(100)
                    x = np.ascontiguousarray(xyz[t])
                    assert L.ref_local_matrix(op_id, order, p, x.ctypes.data, kappa[t], c, buf.ctypes.data) == 0
                    mats[t] = buf[:nb * nb].reshape(nb, nb)
                out[f"m_{op}_{order}_{p}"] = mats
    np.savez_compressed(os.path.join(HERE, "ref_elements.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_elements.npz"))


if __name__ == "__main__":
    main()
