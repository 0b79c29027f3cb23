"""Synthetic deformed-box meshes: the caller-side data the solve path consumes.

In Nek5000 these arrays come from the setup sequence (GLL nodes and D from
core/speclib.f via genwz, geometric factors from core/coef.f glmapm1 /
geodat1, global numbering from core/navier8.f set_vert, masks from
core/bdry.f bcmask, multiplicity from core/connect1.f:126-135, inverse mass
from core/coef.f setinvm).  This module produces the same quantities for a
box of kx*ky*kz hexahedra on the unit cube, vectorised with numpy, so that
benchmarks and users can feed the GPU library without a Nek5000 build:

  * GLL nodes by Golub-Welsch on the Jacobi(1,1) recurrence plus Newton
    polish on the Legendre recurrence; weights 2/(N(N+1) P_N(z)^2);
    D_ij = P_N(z_i) / (P_N(z_j)(z_i - z_j)), D_00 = -N(N+1)/4, D_NN = N(N+1)/4.
  * trilinear element map, then the smooth deformation
    x -> x + amp*sin(pi x) sin(pi y) sin(pi z) * v with one unit vector v per
    mesh (it keeps every face of the cube fixed, so periodic faces match).
  * global ids = lattice index of the GLL node (periodic directions wrap);
    element-interior nodes get id 0, as the reference's set_vert does.

Element e = ex + kx*(ey + ky*ez); point p = ix + lx1*(iy + lx1*iz).
"""
from __future__ import annotations

import math

import numpy as np


def legendre(z, n):
    """P_n(z) by the three-term recurrence."""
    z = np.asarray(z, dtype=np.float64)
    p0, p1 = np.ones_like(z), z.copy()
    if n == 0:
        return p0
    for k in range(1, n):
        p0, p1 = p1, ((2 * k + 1) * z * p1 - k * p0) / (k + 1)
    return p1


def gll(n_points: int):
    """GLL nodes and weights on [-1, 1] (n_points = N+1)."""
    N = n_points - 1
    if N < 1:
        raise ValueError("need at least 2 GLL points")
    if N == 1:
        z = np.array([-1.0, 1.0])
    else:
        # interior nodes: zeros of P'_N = zeros of the Jacobi(1,1) polynomial
        # of degree N-1; Golub-Welsch on its symmetric recurrence matrix.
        k = np.arange(1, N - 1, dtype=np.float64)
        off = np.sqrt(k * (k + 2) / ((2 * k + 1) * (2 * k + 3)))
        J = np.diag(off, 1) + np.diag(off, -1)
        zi = np.sort(np.linalg.eigvalsh(J)) if N > 2 else np.array([0.0])
        # Newton on P'_N using (1-z^2) P'_N = N (P_{N-1} - z P_N)
        for _ in range(4):
            pn = legendre(zi, N)
            pm = legendre(zi, N - 1)
            dp = N * (pm - zi * pn) / (1 - zi * zi)
            # d/dz P'_N = (2 z P'_N - N(N+1) P_N) / (1 - z^2)
            ddp = (2 * zi * dp - N * (N + 1) * pn) / (1 - zi * zi)
            zi = zi - dp / ddp
        z = np.concatenate([[-1.0], zi, [1.0]])
    w = 2.0 / (N * (N + 1) * legendre(z, N) ** 2)
    return z, w


def deriv_matrix(z):
    """Derivative matrix of the Lagrange basis on the GLL nodes z."""
    n = len(z)
    N = n - 1
    pz = legendre(z, N)
    D = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            if i != j:
                D[i, j] = pz[i] / (pz[j] * (z[i] - z[j]))
    D[0, 0] = -N * (N + 1) / 4.0
    D[N, N] = N * (N + 1) / 4.0
    return D


def unit_vector(seed: int):
    """The mesh's deformation direction: a seeded uniform unit vector."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(3)
    return v / np.linalg.norm(v)


def geometry(x, y, z, D, w):
    """Geometric factors of elements given their GLL coordinates x, y, z
    (each (nel, lx1, lx1, lx1), x index fastest): G1..G6 as (6, n), the mass
    bm1 and the Jacobian (core/coef.f glmapm1 / geodat1)."""
    nel, nx = x.shape[0], x.shape[-1]
    zc = z
    # reference-element derivatives: r along ix (last axis), s along iy, t along iz
    def dr(f):
        return np.einsum("il,ekjl->ekji", D, f, optimize=True)

    def ds(f):
        return np.einsum("jl,ekli->ekji", D, f, optimize=True)

    def dt(f):
        return np.einsum("kl,elji->ekji", D, f, optimize=True)

    xr, yr, zr = dr(x), dr(y), dr(zc)
    xs, ys, zs = ds(x), ds(y), ds(zc)
    xt, yt, zt = dt(x), dt(y), dt(zc)
    jac = (xr * (ys * zt - yt * zs) - xs * (yr * zt - yt * zr) + xt * (yr * zs - ys * zr))
    # cofactors (rows of J * grad r, grad s, grad t)
    rx, ry, rz = ys * zt - yt * zs, xt * zs - xs * zt, xs * yt - xt * ys
    sx, sy, sz = yt * zr - yr * zt, xr * zt - xt * zr, xt * yr - xr * yt
    tx, ty, tz = yr * zs - ys * zr, xs * zr - xr * zs, xr * ys - xs * yr
    del xr, yr, zr, xs, ys, zs, xt, yt, zt
    w3 = (w[None, None, :] * w[None, :, None] * w[:, None, None])[None]
    wj = w3 / jac
    g = np.empty((6, nel, nx, nx, nx))
    g[0] = (rx * rx + ry * ry + rz * rz) * wj
    g[1] = (sx * sx + sy * sy + sz * sz) * wj
    g[2] = (tx * tx + ty * ty + tz * tz) * wj
    g[3] = (rx * sx + ry * sy + rz * sz) * wj
    g[4] = (rx * tx + ry * ty + rz * tz) * wj
    g[5] = (sx * tx + sy * ty + sz * tz) * wj
    del rx, ry, rz, sx, sy, sz, tx, ty, tz
    bm1 = (jac * w3).reshape(-1)
    if np.any(jac <= 0):
        raise ValueError("non-positive Jacobian: the element map is tangled")
    return g.reshape(6, -1), bm1, jac.reshape(-1)


def box_mesh(N: int, kx: int, ky: int, kz: int, periodic=(False, False, False),
             dirichlet=None, amp: float = 0.05, v=None, seed: int = 0):
    """Build the operator data for a deformed box.

    Returns a dict with lx1, nel, n, D (lx1,lx1), g (6,n), bm1, glo_num (int64),
    mask, mult, binv, vol, and x, y, z.  dirichlet: flags of the 6 cube faces
    (x-, x+, y-, y+, z-, z+); default: every non-periodic face.
    """
    if periodic[0]:
        raise ValueError("periodic x is not supported")
    nx = N + 1
    nel = kx * ky * kz
    n = nx ** 3 * nel
    z, w = gll(nx)
    D = deriv_matrix(z)
    if v is None:
        v = unit_vector(seed)
    v = np.asarray(v, dtype=np.float64)
    e = np.arange(nel)
    ex, ey, ez = e % kx, (e // kx) % ky, e // (kx * ky)
    h0, h1 = 0.5 * (1.0 - z), 0.5 * (1.0 + z)
    # coordinates (nel, iz, iy, ix)
    xa, xb = ex / kx, (ex + 1) / kx
    ya, yb = ey / ky, (ey + 1) / ky
    za, zb = ez / kz, (ez + 1) / kz
    X = (xa[:, None] * h0[None, :] + xb[:, None] * h1[None, :])[:, None, None, :]
    Y = (ya[:, None] * h0[None, :] + yb[:, None] * h1[None, :])[:, None, :, None]
    Z = (za[:, None] * h0[None, :] + zb[:, None] * h1[None, :])[:, :, None, None]
    X, Y, Z = np.broadcast_arrays(X, Y, Z)
    s = amp * np.sin(math.pi * X) * np.sin(math.pi * Y) * np.sin(math.pi * Z)
    x = X + s * v[0]
    y = Y + s * v[1]
    zc = Z + s * v[2]
    del X, Y, Z, s
    g, bm1, jac = geometry(x, y, zc, D, w)
    # global lattice ids
    ngx = kx * N + 1
    ngy = ky * N + (0 if periodic[1] else 1)
    ngz = kz * N + (0 if periodic[2] else 1)
    ii = np.arange(nx)
    I = (ex[:, None] * N + ii[None, :])[:, None, None, :]
    J = (ey[:, None] * N + ii[None, :])[:, None, :, None]
    K = (ez[:, None] * N + ii[None, :])[:, :, None, None]
    if periodic[1]:
        J = J % ngy
    if periodic[2]:
        K = K % ngz
    lat = (I + ngx * (J + ngy * K)).astype(np.int64)
    lat = np.broadcast_to(lat, (nel, nx, nx, nx)).reshape(-1)
    inner = np.zeros((nx, nx, nx), dtype=bool)
    inner[1:-1, 1:-1, 1:-1] = True
    interior = np.broadcast_to(inner[None], (nel, nx, nx, nx)).reshape(-1)
    glo = np.where(interior, 0, lat + 1).astype(np.int64)
    nglob = ngx * ngy * ngz
    count = np.bincount(lat, minlength=nglob)
    mult = 1.0 / count[lat]
    bsum = np.bincount(lat, weights=bm1, minlength=nglob)
    binv = 1.0 / bsum[lat]
    if dirichlet is None:
        dirichlet = (True, True, not periodic[1], not periodic[1], not periodic[2],
                     not periodic[2])
    Ib = np.broadcast_to(I, (nel, nx, nx, nx)).reshape(-1)
    Jb = np.broadcast_to(J, (nel, nx, nx, nx)).reshape(-1)
    Kb = np.broadcast_to(K, (nel, nx, nx, nx)).reshape(-1)
    mask = np.ones(n)
    if dirichlet[0]:
        mask[Ib == 0] = 0.0
    if dirichlet[1]:
        mask[Ib == ngx - 1] = 0.0
    if dirichlet[2] and not periodic[1]:
        mask[Jb == 0] = 0.0
    if dirichlet[3] and not periodic[1]:
        mask[Jb == ngy - 1] = 0.0
    if dirichlet[4] and not periodic[2]:
        mask[Kb == 0] = 0.0
    if dirichlet[5] and not periodic[2]:
        mask[Kb == ngz - 1] = 0.0
    return dict(lx1=nx, nel=nel, n=n, kx=kx, ky=ky, kz=kz, D=D, zgll=z, wgll=w,
                g=g.reshape(6, n), bm1=bm1, glo_num=glo, mask=mask, mult=mult, binv=binv,
                vol=float(bm1.sum()), x=x.reshape(-1), y=y.reshape(-1), z=zc.reshape(-1),
                lattice=lat, periodic=tuple(periodic))


def face_mask(M, dirichlet):
    """The mask of box_mesh's mesh M for another set of Dirichlet faces
    (x-, x+, y-, y+, z-, z+), e.g. per velocity component."""
    N = M["lx1"] - 1
    per = M.get("periodic", (False, False, False))
    ngx = M["kx"] * N + 1
    ngy = M["ky"] * N + (0 if per[1] else 1)
    ngz = M["kz"] * N + (0 if per[2] else 1)
    lat = M["lattice"]
    I, J, K = lat % ngx, (lat // ngx) % ngy, lat // (ngx * ngy)
    mask = np.ones(M["n"])
    for flag, on, sel in ((dirichlet[0], True, I == 0), (dirichlet[1], True, I == ngx - 1),
                          (dirichlet[2], not per[1], J == 0),
                          (dirichlet[3], not per[1], J == ngy - 1),
                          (dirichlet[4], not per[2], K == 0),
                          (dirichlet[5], not per[2], K == ngz - 1)):
        if flag and on:
            mask[sel] = 0.0
    return mask


def dssum_host(lattice, u, nglob=None):
    """Host direct-stiffness sum by lattice id (harness helper)."""
    s = np.bincount(lattice, weights=u, minlength=nglob or 0)
    return s[lattice]
