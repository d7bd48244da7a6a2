"""CPU oracle pinned against the reference's known-answer test and the
third-party fixtures (no GPU)."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import oracle
from tapkee_gb300 import datasets


def _line_kat(idx, N, k):
    """Port of test/unit/neighbors.cpp:92-127 (BruteKernelNeighbors) assertions."""
    for i in range(N):
        row = list(idx[i])
        assert len(row) == k
        s = set(row)
        assert len(s) == k, "repeated neighbours"
        assert i not in s, "a point is its own neighbour"
        k_left = min(i, k // 2)
        k_right = min(N - i - 1, k // 2)
        for j in range(k_left):
            assert i - j - 1 in s
        for j in range(k_right):
            assert i + j + 1 in s


def test_oracle_line_known_answer():
    N, k = 100, 10
    X = np.arange(N, dtype=np.float64).reshape(N, 1)
    idx, k_used = oracle.find_neighbors(X, k, check_connectivity=True)
    assert k_used == k
    _line_kat(idx, N, k)


def test_oracle_knn_matches_golden(golden):
    X = datasets.swiss_roll(2000, seed=0)
    idx, _, cnt = oracle.knn_brute(X, 12)
    assert (cnt == 12).all()
    assert np.array_equal(idx, golden["lle_idx_oracle_order"])


def test_oracle_weights_vs_sklearn_fixture(golden):
    X = datasets.swiss_roll(2000, seed=0)
    idx = golden["lle_idx_oracle_order"]
    W = oracle.lle_weights(X, idx, 1e-3)
    assert np.abs(W - golden["lle_W"]).max() < 1e-12
    assert np.abs(W - golden["lle_W_sklearn"]).max() / np.abs(W).max() < 1e-9
    assert np.allclose(W.sum(1), 1.0, atol=1e-12)


def test_oracle_assembly_equals_scipy_algebra(golden):
    X = datasets.swiss_roll(2000, seed=0)
    idx = golden["lle_idx_oracle_order"]
    W = golden["lle_W"]
    N, k = idx.shape
    rp, col, vals = oracle.assemble(0, idx, W, 1e-9)
    M = sp.csr_matrix((vals, col, rp), shape=(N, N)).toarray()
    Wm = sp.csr_matrix((W.ravel(), idx.ravel(), np.arange(0, N * k + 1, k)), shape=(N, N))
    IW = sp.eye(N) - Wm
    ref = (IW.T @ IW).toarray() + 1e-9 * np.eye(N)
    assert np.abs(M - ref).max() < 1e-12
    assert int(rp[-1]) == int(golden["lle_nnz"])
    # CSR columns ascending per row; M symmetric
    for r in range(0, N, 97):
        c = col[rp[r]:rp[r + 1]]
        assert np.all(np.diff(c) > 0)
    assert np.abs(M - M.T).max() == 0.0


def _angles(A, B):
    qa, _ = np.linalg.qr(A)
    qb, _ = np.linalg.qr(B)
    s = np.linalg.svd(qa.T @ qb, compute_uv=False)
    return np.arccos(np.clip(s, -1, 1))


def test_oracle_lle_embedding_vs_sklearn_fixture(golden):
    E = golden["lle_embedding"]
    assert _angles(E, golden["lle_embedding_sklearn"]).max() < 1e-4


def test_oracle_dense_eigen_path_vs_shift_invert_lanczos(golden):
    """The eigen step of the oracle (the reference's dense path,
    routines/eigendecomposition.hpp:56-87) on the C1 operator: the golden embedding,
    and the same subspace as scipy's shift-invert Lanczos (ARPACK "SM" through a
    sparse LU, the family of the reference's default Arpack path)."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    sp = pytest.importorskip("scipy.sparse")
    X = datasets.swiss_roll(2000, seed=0)
    idx = golden["lle_idx"]
    W = oracle.lle_weights(X, idx, 1e-3)
    rp, col, vals = oracle.assemble(0, idx, W, 1e-9)
    E, lam = oracle.dense_embedding(rp, col, vals, 2)
    assert _angles(E, golden["lle_embedding"]).max() < 1e-6
    M = sp.csr_matrix((vals, col, rp), shape=(2000, 2000))
    w, V = sla.eigsh(M, k=3, sigma=0, which="LM")
    o = np.argsort(w)
    assert _angles(E, V[:, o[1:3]]).max() < 1e-4
    assert np.allclose(lam, w[o[1:3]], rtol=1e-6, atol=1e-15)


def test_oracle_dense_eigen_known_answer():
    """The reference's sparse smallest-eigenvector known answer
    (test/unit/eigendecomposition.cpp:30-50): M = diag(1, 2, 3) from triplets,
    SmallestEigenvalues with one vector after the skipped one gives the
    eigenvalue 2 and a vector v with |M v - 2 v| ~ 0."""
    rp = np.array([0, 1, 2, 3], np.int64)
    col = np.array([0, 1, 2], np.int32)
    vals = np.array([1.0, 2.0, 3.0])
    E, lam = oracle.dense_embedding(rp, col, vals, 1)
    assert E.shape == (3, 1) and lam.shape == (1,)
    assert abs(lam[0] - 2.0) < 1e-7
    M = np.diag(vals)
    assert np.linalg.norm(M @ E[:, 0] - lam[0] * E[:, 0]) < 1e-7


def test_oracle_ltsa_vs_sklearn_fixture(golden):
    Xs = datasets.lifted_s_curve(1500, d=8, seed=11, noise=0.02, dtype=np.float64)
    idx = golden["ltsa_idx_oracle_order"]
    V = oracle.ltsa_basis(Xs, idx, 2)
    P = np.einsum("nat,nbt->nab", V, V)
    Pg = np.einsum("nat,nbt->nab", golden["ltsa_V"], golden["ltsa_V"])
    assert np.abs(P - Pg).max() < 1e-10
    rp, col, vals = oracle.assemble(1, idx, V, 1e-9)
    assert int(rp[-1]) == int(golden["ltsa_nnz"])
    assert _angles(golden["ltsa_embedding"], golden["ltsa_embedding_sklearn"]).max() < 1e-4


def test_oracle_ltsa_projector_is_orthogonal_projector():
    Xs = datasets.lifted_s_curve(600, d=6, seed=2, noise=0.01, dtype=np.float64)
    idx, _, _ = oracle.knn_brute(Xs, 10)
    V = oracle.ltsa_basis(Xs, idx, 2)
    G = np.concatenate([np.full((600, 10, 1), 1 / np.sqrt(10)), V], axis=2)
    GtG = np.einsum("nat,nas->nts", G, G)
    assert np.abs(GtG - np.eye(3)).max() < 1e-10


def test_oracle_connectivity_retry_two_clusters():
    rng = np.random.default_rng(0)
    a = rng.normal(size=(60, 2))
    b = rng.normal(size=(60, 2)) + 100.0
    X = np.concatenate([a, b])
    idx, _, _ = oracle.knn_brute(X, 5)
    assert not oracle.is_connected(idx)
    idx2, k_used = oracle.find_neighbors(X, 5)
    # 5 -> 10 -> 20 -> 40 -> 80: the first k that reaches across the clusters
    assert k_used > 5 and oracle.is_connected(idx2)


def test_oracle_k_clamped_to_n_minus_one():
    X = np.arange(8, dtype=np.float64).reshape(8, 1)
    idx, k_used = oracle.find_neighbors(X, 50)
    assert k_used == 7 and idx.shape == (8, 7)


@pytest.mark.parametrize("n", [2, 3, 17])
def test_oracle_small_inputs(n):
    X = np.random.default_rng(n).normal(size=(n, 3))
    idx, _, cnt = oracle.knn_brute(X, n - 1)
    for i in range(n):
        assert set(idx[i]) == set(range(n)) - {i}


def _hlle_blocks_np(X, idx, td, flip=None):
    """Donoho-Grimes Hessian blocks from an SVD tangent basis and a Householder
    QR; flip multiplies the basis columns by +-1."""
    k = idx.shape[1]
    dp = td * (td + 1) // 2
    out = np.zeros((len(idx), k, k))
    for i in range(len(idx)):
        G = X[idx[i]] - X[idx[i]].mean(0)
        U = np.linalg.svd(G, full_matrices=False)[0][:, :td]
        if flip is not None:
            U = U * flip
        cols = [np.ones(k)] + [U[:, t] for t in range(td)]
        cols += [U[:, j] * U[:, l] for j in range(td) for l in range(j, td)]
        H = np.linalg.qr(np.stack(cols, 1))[0][:, 1 + td:1 + td + dp]
        S = H.sum(0)
        H = H / np.where(S > 1e-4, S, 1.0)
        out[i] = H @ H.T
    return out


def test_oracle_hessian_vs_fixture(golden):
    """hessian_weight_matrix (routines/locally_linear.hpp:161-255) on the
    lifted S-curve: the committed blocks, nnz, M checksum and embedding."""
    Xs = datasets.lifted_s_curve(1500, d=8, seed=11, noise=0.02, dtype=np.float64)
    idx = golden["ltsa_idx_oracle_order"]
    B = oracle.hessian_blocks(Xs, idx, 2)
    assert np.abs(B[:64] - golden["hlle_B"]).max() < 1e-12
    rp, col, vals = oracle.assemble(2, idx, B, 0.0)
    assert int(rp[-1]) == int(golden["hlle_nnz"])
    assert abs(np.abs(vals).sum() - golden["hlle_M_checksum"]) < 1e-9 * golden["hlle_M_checksum"]
    E, lam = oracle.dense_embedding(rp, col, vals, 2)
    assert _angles(E, golden["hlle_embedding"]).max() < 1e-6
    assert _angles(golden["hlle_embedding"], golden["hlle_embedding_numpy"]).max() < 1e-6
    # not the LTSA embedding of the same neighbourhoods
    assert _angles(E, golden["ltsa_embedding"]).max() > 1e-2


def test_oracle_hessian_block_is_a_sign_free_projector():
    """Every column of the Gram-Schmidt basis after the constant one sums to
    zero, so the column-sum division (routines/locally_linear.hpp:226-231) does
    not fire and B is the orthogonal projector onto the quadratic part, rank
    td (td + 1) / 2: independent of the eigenvector signs and of how the
    tangent basis was computed."""
    Xs = datasets.lifted_s_curve(400, d=6, seed=4, noise=0.01, dtype=np.float64)
    idx, _, _ = oracle.knn_brute(Xs, 10)
    for td in (1, 2):
        B = oracle.hessian_blocks(Xs, idx, td)
        dp = td * (td + 1) // 2
        assert np.abs(np.einsum("nab,nbc->nac", B, B) - B).max() < 1e-12
        assert np.abs(np.trace(B, axis1=1, axis2=2) - dp).max() < 1e-12
        assert np.abs(B.sum(2)).max() < 1e-12
        V = oracle.ltsa_basis(Xs, idx, td)
        assert np.abs(np.einsum("nab,nbt->nat", B, V)).max() < 1e-12
        for flip in ([1.0] * td, [-1.0] + [1.0] * (td - 1), [-1.0] * td):
            assert np.abs(B - _hlle_blocks_np(Xs, idx, td, np.array(flip))).max() < 1e-9
    with pytest.raises(ValueError):
        oracle.hessian_blocks(Xs, idx, 3)
