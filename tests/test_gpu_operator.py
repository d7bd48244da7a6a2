"""The whole stage (tk_local_operator) vs the oracle, plus the reference's error
semantics (test/unit/interface.cpp) on the GPU path."""
import numpy as np
import pytest

import tapkee_gb300 as tk
from oracle import oracle
from tapkee_gb300 import datasets

pytestmark = pytest.mark.gpu


def _angles(A, B):
    qa, _ = np.linalg.qr(A)
    qb, _ = np.linalg.qr(B)
    return np.arccos(np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False), -1, 1))


@pytest.mark.parametrize("screen", ["tensor", "fp32"])
def test_lle_operator_and_embedding(ctx, golden, screen):
    X = datasets.swiss_roll(2000, seed=0)
    op = ctx.local_operator(X, "lle", num_neighbors=12, klle_shift=1e-3, screen=screen)
    assert np.array_equal(op.idx, golden["lle_idx"])
    W_ref = oracle.lle_weights(X, op.idx, 1e-3)
    assert np.abs(op.weights - W_ref).max() / np.abs(W_ref).max() < 1e-5
    rp, col, vals = oracle.assemble(0, op.idx, W_ref, 1e-9)
    assert np.array_equal(op.row_ptr, rp) and np.array_equal(op.col_idx, col)
    assert np.abs(op.vals - vals).max() / np.abs(vals).max() < 1e-5
    E, _ = tk.smallest_eigenvectors(op, 2)
    assert _angles(E, golden["lle_embedding"]).max() < 1e-4


def test_ltsa_operator_and_embedding(ctx, golden):
    X = datasets.lifted_s_curve(1500, d=8, seed=11, noise=0.02, dtype=np.float64)
    op = ctx.local_operator(X, "ltsa", num_neighbors=12, target_dimension=2)
    ref_idx = golden["ltsa_idx_oracle_order"]
    assert all(set(a) == set(b) for a, b in zip(op.idx.tolist(), ref_idx.tolist()))
    V_ref = oracle.ltsa_basis(X, op.idx, 2)
    P = np.einsum("nat,nbt->nab", op.weights, op.weights)
    Pr = np.einsum("nat,nbt->nab", V_ref, V_ref)
    assert np.abs(P - Pr).max() < 1e-5
    E, _ = tk.smallest_eigenvectors(op, 2)
    assert _angles(E, golden["ltsa_embedding"]).max() < 1e-4


def test_embed_and_chain_entry_points(ctx, golden):
    X = datasets.swiss_roll(2000, seed=0)
    E1 = tk.embed(X.T, method="lle", neighbors_method="brute", num_neighbors=12, klle_shift=1e-3, context=ctx)
    assert E1.shape == (2000, 2)
    assert _angles(E1, golden["lle_embedding"]).max() < 1e-4
    out = tk.with_(method="lle", neighbors_method="brute", num_neighbors=12, klle_shift=1e-3).embed_using(
        X.T, context=ctx)
    assert _angles(out.embedding, golden["lle_embedding"]).max() < 1e-4


def test_connectivity_retry_matches_oracle(ctx):
    rng = np.random.default_rng(0)
    X = np.concatenate([rng.normal(size=(60, 2)), rng.normal(size=(60, 2)) + 100.0])
    msgs = []
    ctx.set_logger(lambda lvl, m: msgs.append((lvl, m)))
    try:
        op = ctx.local_operator(X, "lle", num_neighbors=5)
    finally:
        ctx.set_logger(None)
    _, k_ref = oracle.find_neighbors(X, 5)
    assert op.k == k_ref and op.connectivity_retries >= 1
    assert any("not connected" in m for _, m in msgs)
    assert ctx.check_connected(op.idx)


def test_reference_error_semantics(ctx):
    X = datasets.swiss_roll(50, seed=1)
    with pytest.raises(tk.WrongParameterError):  # interface.cpp:144-158
        ctx.local_operator(X, "lle", num_neighbors=-3)
    with pytest.raises(tk.WrongParameterError):  # num_neighbors must be < N
        ctx.local_operator(X, "lle", num_neighbors=50)
    with pytest.raises(tk.WrongParameterError):  # methods/base.hpp:44
        ctx.local_operator(X, "lle", num_neighbors=5, target_dimension=50)
    with pytest.raises(tk.NoDataError):  # interface.cpp:102-119
        ctx.local_operator(np.zeros((0, 3)), "lle")
    with pytest.raises(tk.CancelledError):  # interface.cpp:176-196
        ctx.local_operator(X, "lle", num_neighbors=5, cancel_function=lambda: True)
    with pytest.raises(tk.UnsupportedMethodError):
        ctx.local_operator(X, "isomap")
    # the context stays usable after errors
    op = ctx.local_operator(X, "lle", num_neighbors=5)
    assert op.idx.shape == (50, 5)
