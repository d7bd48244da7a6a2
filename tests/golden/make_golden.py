"""Generates the golden fixtures under tests/golden/ (run once, results committed).

    python tests/golden/make_golden.py

The reference (lisitsyn/tapkee) cannot be built here (it needs Eigen), so the
fixtures come from the CPU oracle (oracle/tapkee_oracle.cpp, a restatement of the
reference's routines) and are cross-checked, at generation time, against
scikit-learn's independent implementations of the same published formulas:

* kNN sets       -- sklearn.neighbors.NearestNeighbors(algorithm="brute"), FP64;
* LLE weights    -- sklearn.manifold._locally_linear.barycenter_weights, which uses
                    the same reg * trace(C) regularisation as
                    routines/locally_linear.hpp:128-129;
* LLE embedding  -- sklearn LocallyLinearEmbedding(method="standard", dense eigh);
* LTSA embedding -- sklearn LocallyLinearEmbedding(method="ltsa", dense eigh);
                    its alignment update equals routines/locally_linear.hpp:65-77
                    without the (i,i,shift) triplet.
* HLLE blocks    -- hlle_blocks_numpy below, the Donoho-Grimes estimator with
                    an SVD tangent basis and a Householder QR (the oracle uses a
                    Jacobi eigenbasis and Gram-Schmidt). scikit-learn's
                    method="hessian" is no cross-check here: it keeps every
                    column of a full QR past 1 + td, so its block is
                    I - P[1, V], the LTSA block, and its embedding equals its
                    LTSA embedding.

The scikit-learn outputs are stored next to the oracle's so the cross-check can
be replayed where scikit-learn is not installed.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from tapkee_gb300 import datasets  # noqa: E402


def sort_rows_by_distance(X, idx):
    """Neighbour rows ordered by (FP64 distance, index)."""
    X = np.asarray(X, np.float64)
    d = ((X[idx] - X[:, None, :]) ** 2).sum(-1)
    order = np.array([np.lexsort((idx[i], d[i])) for i in range(len(idx))])
    return np.take_along_axis(idx, order, 1)


def principal_angles(A, B):
    qa, _ = np.linalg.qr(A)
    qb, _ = np.linalg.qr(B)
    s = np.linalg.svd(qa.T @ qb, compute_uv=False)
    return np.arccos(np.clip(s, -1, 1))


def hlle_blocks_numpy(X, idx, td):
    """Hessian blocks B_i = H H^T, H the dp product columns of the reduced QR of
    [1, U, U_j U_l] (U: top-td left singular vectors of the centred neighbours),
    a product column divided by its sum when that sum exceeds 1e-4."""
    k = idx.shape[1]
    dp = td * (td + 1) // 2
    out = np.zeros((len(idx), k, k))
    for i in range(len(idx)):
        G = X[idx[i]] - X[idx[i]].mean(0)
        U = np.linalg.svd(G, full_matrices=False)[0][:, :td]
        cols = [np.ones(k)] + [U[:, t] for t in range(td)]
        cols += [U[:, j] * U[:, l] for j in range(td) for l in range(j, td)]
        Q = np.linalg.qr(np.stack(cols, 1))[0]
        H = Q[:, 1 + td:1 + td + dp]
        S = H.sum(0)
        H = H / np.where(S > 1e-4, S, 1.0)
        out[i] = H @ H.T
    return out


def main():
    from sklearn.manifold import LocallyLinearEmbedding
    from sklearn.manifold._locally_linear import barycenter_weights
    from sklearn.neighbors import NearestNeighbors

    out = {}
    # ---- LLE on the Swiss roll, N=2000, D=3, k=12, klle_shift=1e-3, td=2 ----
    X = datasets.swiss_roll(2000, seed=0)
    k, shift, td = 12, 1e-3, 2
    idx, dist, cnt = oracle.knn_brute(X, k)
    assert (cnt == k).all()
    assert oracle.is_connected(idx)
    nn = NearestNeighbors(n_neighbors=k + 1, algorithm="brute").fit(X)
    sk_idx = nn.kneighbors(X, return_distance=False)[:, 1:]
    assert all(set(a) == set(b) for a, b in zip(idx, sk_idx)), "kNN sets differ from sklearn"
    W = oracle.lle_weights(X, idx, shift)
    W_sk = barycenter_weights(X, X, idx, reg=shift)
    werr = np.abs(W - W_sk).max() / np.abs(W_sk).max()
    assert werr < 1e-9, werr
    rp, col, vals = oracle.assemble(0, idx, W, 1e-9)
    E, ev = oracle.dense_embedding(rp, col, vals, td)
    lle = LocallyLinearEmbedding(n_neighbors=k, n_components=td, reg=shift, eigen_solver="dense",
                                 method="standard")
    E_sk = lle.fit_transform(X)
    ang = principal_angles(E, E_sk).max()
    assert ang < 1e-4, ang
    out.update(lle_idx=sort_rows_by_distance(X, idx), lle_W_sklearn=W_sk, lle_idx_oracle_order=idx,
               lle_W=W, lle_embedding=E, lle_embedding_sklearn=E_sk, lle_evals=ev,
               lle_nnz=np.int64(rp[-1]), lle_M_checksum=np.float64(np.abs(vals).sum()))
    print(f"LLE: W vs sklearn {werr:.2e}, embedding angle vs sklearn {ang:.2e}, nnz {rp[-1]}")

    # ---- LTSA on the S-curve lifted to D=8, N=1500, k=12, td=2 ----
    Xs = datasets.lifted_s_curve(1500, d=8, seed=11, noise=0.02, dtype=np.float64)
    k2 = 12
    idx2, _, cnt2 = oracle.knn_brute(Xs, k2)
    assert (cnt2 == k2).all()
    V, evl = oracle.ltsa_basis(Xs, idx2, td, return_evals=True)
    rp2, col2, vals2 = oracle.assemble(1, idx2, V, 1e-9)
    E2, _ = oracle.dense_embedding(rp2, col2, vals2, td)
    ltsa = LocallyLinearEmbedding(n_neighbors=k2, n_components=td, eigen_solver="dense", method="ltsa")
    E2_sk = ltsa.fit_transform(Xs)
    ang2 = principal_angles(E2, E2_sk).max()
    assert ang2 < 1e-4, ang2
    out.update(ltsa_idx_oracle_order=idx2, ltsa_V=V, ltsa_embedding=E2,
               ltsa_embedding_sklearn=E2_sk, ltsa_nnz=np.int64(rp2[-1]))
    print(f"LTSA: embedding angle vs sklearn {ang2:.2e}, nnz {rp2[-1]}")

    # ---- Hessian LLE on the same S-curve, k=12, td=2 ----
    B = oracle.hessian_blocks(Xs, idx2, td)
    B_np = hlle_blocks_numpy(Xs, idx2, td)
    berr = np.abs(B - B_np).max()
    assert berr < 1e-9, berr
    rp3, col3, vals3 = oracle.assemble(2, idx2, B, 0.0)
    E3, ev3 = oracle.dense_embedding(rp3, col3, vals3, td)
    rp4, col4, vals4 = oracle.assemble(2, idx2, B_np, 0.0)
    E3_np, _ = oracle.dense_embedding(rp4, col4, vals4, td)
    ang3 = principal_angles(E3, E3_np).max()
    assert ang3 < 1e-6, ang3
    out.update(hlle_B=B[:64], hlle_embedding=E3, hlle_embedding_numpy=E3_np,
               hlle_evals=ev3, hlle_nnz=np.int64(rp3[-1]), hlle_M_checksum=np.float64(np.abs(vals3).sum()))
    print(f"HLLE: blocks vs numpy {berr:.2e}, embedding angle vs numpy {ang3:.2e}, evals {ev3}, nnz {rp3[-1]}")

    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **out)
    print("wrote", os.path.join(HERE, "golden_small.npz"))


if __name__ == "__main__":
    main()
