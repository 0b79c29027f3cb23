"""The library's host setup of the pressure preconditioner (h1mg_plan.cpp,
through the host-only entry points of nekmesh.h) against the oracle's
restatement: level orders, face types, masks, restriction and Schwarz
weights, element widths and the 1-D fast-diagonalisation operators.  No GPU
is touched."""
import numpy as np
import pytest

from conftest import rng_unit_vector

from nek5000_gb300 import meshio


def test_levels_match(oracle):
    for lx in range(3, 13):
        assert meshio.h1mg_levels(lx) == oracle.h1mg_levels(lx), lx


def _cases(oracle):
    return [
        oracle.box_problem(6, 3, 3, 2, v=rng_unit_vector(101)),
        oracle.box_problem(5, 3, 4, 3, periodic=(False, True, True), v=rng_unit_vector(102)),
        oracle.box_problem(8, 2, 3, 2, dirichlet=(True, False, False, True, False, False),
                           v=rng_unit_vector(103)),
        oracle.box_problem(4, 3, 3, 3, dirichlet=(False,) * 6, v=rng_unit_vector(104)),
    ]


def test_face_types_match(oracle):
    for P in _cases(oracle):
        want = oracle.face_types(P["nx1"], P["nel"], P["glo_num"], P["mask"])
        got = meshio.face_types(P["nx1"], P["glo_num"], P["mask"])
        assert np.array_equal(got, want)


def test_level_setup_matches(oracle):
    """Masks, restriction and Schwarz weights equal the oracle's exactly;
    element widths to 1e-13 (the GLL points come from different codes)."""
    for P in _cases(oracle):
        fbc = oracle.face_types(P["nx1"], P["nel"], P["glo_num"], P["mask"])
        mg = oracle.H1mg(P["ops"], P["x"], P["y"], P["z"], fbc, P["vertex"])
        for l, nxl in enumerate(mg.levels):
            nx, mask, rwt, swt, lengths = meshio.h1mg_level(P["nx1"], P["glo_num"], P["x"],
                                                            P["y"], P["z"], l, mask=P["mask"])
            omask, orwt, oswt = mg.level(l)
            assert nx == nxl
            assert np.array_equal(mask, omask), l
            assert np.array_equal(rwt, orwt), l
            assert np.array_equal(swt, oswt), l
        assert np.allclose(lengths, mg.lengths(), rtol=1e-13, atol=0)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 11])
@pytest.mark.parametrize("lbc,rbc", [(0, 0), (0, 1), (2, 0), (1, 2), (2, 2), (1, 1)])
def test_fdm1d_matches(oracle, n, lbc, rbc):
    """The same operator S diag(lam) S^T (basis-independent) and the same
    eigenvalues; S is B-orthonormal (S^T B S = I on the kept rows)."""
    ll, lm, lr = 0.7, 1.1, 0.9
    S, lam = meshio.fdm1d(n, lbc, rbc, ll, lm, lr)
    So, lamo = oracle.fdm1d(n, lbc, rbc, ll, lm, lr)
    assert np.allclose(lam, lamo, rtol=1e-12, atol=1e-13 * np.abs(lamo).max())
    inv = lambda v: np.where(np.abs(v) > 1e-8 * np.abs(v).max(), 1.0 / np.where(v == 0, 1, v), 0)
    M = S @ np.diag(inv(lam)) @ S.T  # the zero mode of a floating 1-D block left out
    Mo = So @ np.diag(inv(lamo)) @ So.T
    assert np.allclose(M, Mo, rtol=0, atol=1e-11 * np.abs(Mo).max())


def test_xxt_factor_inverts_and_stays_sparse():
    """X X^T = A^-1 for the 27-point vertex operator of a 12^3 box (random
    SPD element matrices), and X has far fewer entries than n^2 with the
    nested-dissection order (columns non-zero only on their subtree)."""
    sp = pytest.importorskip("scipy.sparse")
    k = 11  # vertices 12^3
    nv = (k + 1) ** 3
    rng = np.random.default_rng(7)
    g = np.arange(nv).reshape(k + 1, k + 1, k + 1)
    rows, cols, vals = [], [], []
    for ez in range(k):
        for ey in range(k):
            for ex in range(k):
                ids = np.array([g[ez + (c >> 2), ey + ((c >> 1) & 1), ex + (c & 1)] for c in range(8)])
                B = rng.standard_normal((8, 8))
                Ae = B @ B.T + 8 * np.eye(8)
                rows.append(np.repeat(ids, 8))
                cols.append(np.tile(ids, 8))
                vals.append(Ae.reshape(-1))
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(nv, nv))
    zz, yy, xx = np.meshgrid(*(np.arange(k + 1.0),) * 3, indexing="ij")
    xyz = np.stack([xx.reshape(-1), yy.reshape(-1), zz.reshape(-1)], axis=1)
    perm, X = meshio.xxt_factor(A, xyz)
    assert sorted(perm.tolist()) == list(range(nv))
    Ap = A.toarray()[np.ix_(perm, perm)]
    assert np.allclose(X @ X.T @ Ap, np.eye(nv), atol=1e-10)
    assert np.count_nonzero(X) < 0.4 * nv * nv
