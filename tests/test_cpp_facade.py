"""The C++ facade include/tapkee_gb300.hpp (tapkee::with(...) chain shape),
compiled with g++ against the in-tree library and run as a program."""
import os
import subprocess

import numpy as np
import pytest

from tapkee_gb300 import datasets

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_check.cpp")
OUT = os.path.join(ROOT, "tests", "cpp", "_build")


@pytest.fixture(scope="module")
def facade_bin():
    from tapkee_gb300 import build as tkbuild
    tkbuild.build()
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "facade_check")
    libdir = os.path.dirname(tkbuild.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", f"-I{os.path.join(ROOT, 'include')}", SRC,
           f"-L{libdir}", "-ltapkee_gb300", f"-Wl,-rpath,{libdir}", "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def test_facade_host_semantics(facade_bin):
    import torch
    if torch.cuda.is_available():
        pytest.skip("checks the no-device path")
    r = subprocess.run([facade_bin, "host"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok"


@pytest.mark.gpu
def test_facade_lle_c1_matches_oracle(facade_bin, golden, tmp_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from oracle import oracle
    X = datasets.swiss_roll(2000, seed=0)
    xpath = tmp_path / "X.bin"
    np.ascontiguousarray(X, dtype=np.float64).tofile(xpath)
    prefix = str(tmp_path / "op_")
    r = subprocess.run([facade_bin, "gpu", str(xpath), "2000", "3", prefix], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    idx = np.fromfile(prefix + "idx.bin", np.int32).reshape(2000, 12)
    W = np.fromfile(prefix + "w.bin", np.float64).reshape(2000, 12)
    rp = np.fromfile(prefix + "rowptr.bin", np.int64)
    col = np.fromfile(prefix + "col.bin", np.int32)
    vals = np.fromfile(prefix + "vals.bin", np.float64)
    assert np.array_equal(idx, golden["lle_idx"])
    W_ref = oracle.lle_weights(X, idx, 1e-3)
    assert np.abs(W - W_ref).max() / np.abs(W_ref).max() < 1e-5
    rp_ref, col_ref, vals_ref = oracle.assemble(0, idx, W_ref, 1e-9)
    assert np.array_equal(rp, rp_ref) and np.array_equal(col, col_ref)
    assert np.abs(vals - vals_ref).max() / np.abs(vals_ref).max() < 1e-5
    # embedUsing: N x 2 column-major embedding, the golden dense-oracle subspace
    E = np.fromfile(prefix + "embedding.bin", np.float64).reshape(2, 2000).T
    qa, _ = np.linalg.qr(E)
    qb, _ = np.linalg.qr(golden["lle_embedding"])
    assert np.arccos(np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False), -1, 1)).max() < 1e-4
