"""The adjoint gradient dJ/dkappa_e = -lambda_e^T Khat_e u_e behind a
torch.autograd.Function (test harness only), and the 64^3 adjoint workload:
J(kappa) = 1/2 ||u(kappa) - u_target||^2, u_target from a lognormal kappa*
(sigma 1), kappa lognormal sigma 0.5 (seed 2), gradient checked against central
finite differences on 64 random elements and against the gradient the oracle
computes from its FP64 element matrices."""
import numpy as np
import pytest

import morganapublic_gb300 as mg
import oracle as orc
from morganapublic_gb300 import meshgen

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)


class Problem:
    """-div(kappa grad u) = 1 on a Kuhn cube, u = 0 on the boundary (symmetric elimination)."""

    def __init__(self, n, jitter=0.0, seed=1, permute=False, rtol=1e-13):
        self.m = meshgen.kuhn_cube(n, jitter=jitter, seed=seed, permute=permute)
        self.mesh = mg.Mesh(self.m.xyz, self.m.conn, order=1)
        self.b = mg.MatrixBuilder(self.mesh)
        self.mask = torch.from_numpy(self.m.boundary)
        self.f = self.b.build_vector(quad=4)
        self.f[self.mask.cuda()] = 0.0
        self.rtol = rtol

    def solve(self, kappa, rhs=None):
        v = self.b.assemble("stiff_kappa", coeff=kappa, quad=4)
        self.b.apply_dirichlet(v, self.mask)
        x, _ = self.b.cg(v, (self.f if rhs is None else rhs).clone(), rtol=self.rtol, maxit=50000)
        return x


class AdjointJ(torch.autograd.Function):
    """J(kappa) = 1/2 ||u(kappa) - u_t||^2; backward: one adjoint solve (the
    operator is symmetric) and the per-element gradient kernel."""

    @staticmethod
    def forward(ctx, kappa, prob, ut):
        u = prob.solve(kappa.detach())
        ctx.prob = prob
        ctx.save_for_backward(kappa, u, ut)
        return 0.5 * ((u - ut) ** 2).sum()

    @staticmethod
    def backward(ctx, gout):
        kappa, u, ut = ctx.saved_tensors
        prob = ctx.prob
        lam = prob.solve(kappa.detach(), rhs=u - ut)
        g = prob.b.adjoint_grad(u, lam, quad=4)
        return gout * g, None, None


def test_autograd_function_gradcheck():
    prob = Problem(2, jitter=0.2, seed=4, permute=True, rtol=1e-14)
    E = len(prob.m.conn)
    kappa = torch.from_numpy(meshgen.lognormal(E, 0.5, 2)).cuda().requires_grad_(True)
    ut = prob.solve(torch.from_numpy(meshgen.lognormal(E, 1.0, 20)).cuda())
    assert torch.autograd.gradcheck(lambda k: AdjointJ.apply(k, prob, ut), (kappa,), eps=1e-6, atol=1e-9, rtol=1e-4)


def test_adjoint_64cube_fd_and_oracle():
    prob = Problem(64, jitter=0.2, seed=2, permute=True)
    m, E = prob.m, len(prob.m.conn)
    kstar = torch.from_numpy(meshgen.lognormal(E, 1.0, 20)).cuda()
    ut = prob.solve(kstar)
    kappa = torch.from_numpy(meshgen.lognormal(E, 0.5, 2)).cuda().requires_grad_(True)
    J = AdjointJ.apply(kappa, prob, ut)
    J.backward()
    g = kappa.grad.cpu().numpy()
    # against the oracle: the same u and lambda through the oracle's FP64 element matrices
    u = prob.solve(kappa.detach())
    lam = prob.solve(kappa.detach(), rhs=u - ut)
    g_ref = orc.adjoint_grad(1, 4, m.xyz, m.conn, prob.mesh.elem_dofs(), u.cpu().numpy(), lam.cpu().numpy())
    assert np.max(np.abs(g - g_ref)) <= 1e-12 * np.abs(g_ref).max()
    # central differences on 64 random elements (h = 1e-2 kappa_e), and along one
    # random direction over all elements (a well-conditioned check of the whole field)
    k0 = kappa.detach().clone()
    Jf = lambda k: 0.5 * float(((prob.solve(k) - ut) ** 2).sum())
    gmax = np.abs(g).max()
    errs = []
    for e in np.random.default_rng(2).choice(E, 64, replace=False):
        h = 1e-2 * float(k0[e])
        kp, km = k0.clone(), k0.clone()
        kp[e] += h
        km[e] -= h
        fd = (Jf(kp) - Jf(km)) / (2 * h)
        errs.append(abs(fd - g[e]) / gmax)
    d = torch.from_numpy(np.random.default_rng(5).uniform(-1, 1, E)).cuda() * k0
    t = 1e-3
    fd_dir = (Jf(k0 + t * d) - Jf(k0 - t * d)) / (2 * t)
    an_dir = float((torch.from_numpy(g).cuda() * d).sum())
    print("adjoint 64^3: worst per-element FD error / max|g| = %.3e, directional rel err = %.3e"
          % (max(errs), abs(fd_dir - an_dir) / abs(an_dir)))
    assert max(errs) <= 1e-5
    assert abs(fd_dir - an_dir) <= 1e-5 * abs(an_dir)
