"""Adjoint of the Helmholtz solve with respect to the per-point viscosity h1.

J(h1) = 0.5 * sum_p bm1_p (u_p - u*_p)^2 with u solving the masked, assembled
system mask * dssum(A(h1) u) = f (h2 = 0).  The gradient is
dJ/dh1 = -axhelm_adjoint_h1(lam, u), lam solving the same (symmetric) system
with right-hand side mask * dssum(bm1 (u - u*)).  It is wrapped in a
torch.autograd.Function here, in the test harness only, and checked
  * against central finite differences of J (eps = 1e-6, 32 random directions);
  * against the exact directional derivative -lam^T A(delta) u built with the
    oracle's axhelm (A is linear in h1).
"""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu

TOL = -1e-12


def gaussian_field(x, y, z, seed, length=0.2, modes=64):
    """Seeded smooth Gaussian random field: random Fourier modes with a
    Gaussian spectrum of correlation length `length`, unit variance."""
    r = np.random.default_rng(seed)
    k = r.standard_normal((modes, 3)) / length
    ph = r.uniform(0, 2 * np.pi, modes)
    a = r.standard_normal(modes) * np.sqrt(2.0 / modes)
    return (a[None, :] * np.cos(np.outer(x, k[:, 0]) + np.outer(y, k[:, 1]) +
                                np.outer(z, k[:, 2]) + ph[None, :])).sum(1)


def make_solver(lib, P, torch):
    dev = lambda a: torch.tensor(a, device="cuda")
    n = P["n"]
    mask, mult, binv = dev(P["mask"]), dev(P["mult"]), dev(P["binv"])
    h2 = torch.zeros(n, dtype=torch.float64, device="cuda")

    def solve(h1, rhs):
        u = torch.zeros(n, dtype=torch.float64, device="cuda")
        it, r0, r2, rc = lib.cggo(u, rhs, h1.contiguous(), h2, mask, mult, 1, TOL, 10 ** 6, 1, binv,
                                  maxcg=10 ** 6)
        assert rc == 0, lib.last_error()
        return u

    class HelmholtzSolve(torch.autograd.Function):
        @staticmethod
        def forward(ctx, h1, f):
            u = solve(h1, f)
            ctx.save_for_backward(h1, u)
            return u

        @staticmethod
        def backward(ctx, gu):
            h1, u = ctx.saved_tensors
            g = gu.detach().contiguous().clone()
            lib.dssum(g)
            g = g * mask
            lam = torch.zeros_like(u)
            it, r0, r2, rc = lib.cggo_adjoint(lam, g, h1.contiguous(), h2, mask, mult, 1, TOL,
                                              10 ** 6, 1, binv, maxcg=10 ** 6)
            assert rc == 0
            gh1 = torch.zeros_like(u)
            lib.axhelm_adjoint_h1(gh1, lam, u)
            return -gh1, None

    return HelmholtzSolve, solve


@pytest.mark.parametrize("shape", [(8, 3, 3, 3), (8, 16, 16, 16)])
def test_adjoint_gradient(gpu_lib, oracle, shape):
    torch = pytest.importorskip("torch")
    nx1, kx, ky, kz = shape
    P = oracle.box_problem(nx1, kx, ky, kz, v=rng_unit_vector(5))
    n = P["n"]
    x, y, z = P["x"], P["y"], P["z"]
    h1 = np.exp(0.3 * gaussian_field(x, y, z, seed=5))
    h1t = np.exp(0.3 * gaussian_field(x, y, z, seed=6)) * h1  # perturbed viscosity for u*
    rng = np.random.default_rng(5)
    f = P["ops"].dssum(P["bm1"] * (P["ops"].dssum(rng.standard_normal(n)) * P["mult"])) * P["mask"]
    lib = gpu_lib(0)
    lib.setup(nx1, P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    Solve, solve = make_solver(lib, P, torch)
    dev = lambda a: torch.tensor(a, device="cuda")
    ft, bm1 = dev(f), dev(P["bm1"])
    ustar = solve(dev(h1t), ft)

    def J(h):
        u = solve(h, ft)
        return 0.5 * float(torch.sum(bm1 * (u - ustar) ** 2))

    h = dev(h1).requires_grad_(True)
    u = Solve.apply(h, ft)
    Jv = 0.5 * torch.sum(bm1 * (u - ustar) ** 2)
    Jv.backward()
    grad = h.grad.detach()
    assert float(grad.abs().max()) > 0
    rngd = np.random.default_rng(7)
    eps = 1e-6
    fd_err, ex_err = [], []
    u_np = u.detach().cpu().numpy()
    ndir = 32  # as the configuration states, at every size
    for q in range(ndir):
        delta = rngd.standard_normal(n) * h1
        dd = dev(delta)
        gd = float(torch.dot(grad, dd))
        jp, jm = J(dev(h1 + eps * delta)), J(dev(h1 - eps * delta))
        fd = (jp - jm) / (2 * eps)
        fd_err.append(abs(fd - gd) / max(abs(fd), 1e-300))
    # exact directional derivative with the oracle's operator: -lam^T A(delta) u
    # (lam recomputed here; the backward pass above computed the same one)
    g = bm1 * (u.detach() - ustar)
    lib.dssum(g)
    g = g * dev(P["mask"])
    lam = torch.zeros_like(u)
    lib.cggo_adjoint(lam, g, dev(h1), torch.zeros_like(u), dev(P["mask"]), dev(P["mult"]), 1, TOL,
                     10 ** 6, 1, dev(P["binv"]), maxcg=10 ** 6)
    lam_np = lam.cpu().numpy()
    for q in range(8):
        delta = rngd.standard_normal(n) * h1
        exact = -float(np.dot(lam_np, P["ops"].axhelm(u_np, delta, np.zeros(n))))
        gd = float(torch.dot(grad, dev(delta)))
        ex_err.append(abs(exact - gd) / abs(exact))
    print(f"adjoint {shape}: FD rel. err max {max(fd_err):.2e} median {np.median(fd_err):.2e}; "
          f"oracle-operator rel. err max {max(ex_err):.2e}")
    assert max(ex_err) < 1e-9
    assert np.median(fd_err) < 1e-5 and max(fd_err) < 1e-3


def test_adjoint_kernel_matches_oracle_operator(gpu_lib, oracle):
    """sum_p gh1_p delta_p = lam^T A(delta) u for arbitrary lam, u, delta."""
    P = oracle.box_problem(6, 2, 3, 2, v=rng_unit_vector(8))
    n = P["n"]
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    r = np.random.default_rng(8)
    lam, u = r.standard_normal(n), r.standard_normal(n)
    gh1 = np.zeros(n)
    lib.axhelm_adjoint_h1(gh1, lam, u)
    for q in range(4):
        delta = r.standard_normal(n)
        exact = float(np.dot(lam, P["ops"].axhelm(u, delta, np.zeros(n))))
        assert abs(np.dot(gh1, delta) - exact) <= 1e-12 * np.sum(np.abs(gh1 * delta))
