"""Command-line entry point in the shape of the reference's `tapkee` tool
(src/cli/main.cpp:156-548) for the methods this library provides.

    python -m tapkee_gb300 -i data.csv -o embedding.csv -m lle -k 10 -td 2

Same option names, defaults and messages as the reference tool where they apply:
  -i/--input-file (default /dev/stdin), -o/--output-file (default /dev/stdout),
  --transpose-input, --transpose-output, -d/--delimiter (","),
  -m/--method ("locally_linear_embedding"), -nm/--neighbors-method,
  -em/--eigen-method ("arpack"), -td/--target-dimension (2),
  -k/--num-neighbors (10), --eigenshift (1e-9), --benchmark, --verbose.
The file is read and written with the tool's delimited-matrix format
(tapkee_gb300.io, src/cli/util.hpp:73-130): a line is one point unless
--transpose-input says the file holds one feature per line (main.cpp:453-458).
As in the tool, check_connectivity is on (main.cpp:481).

Methods: KLLE, KLTSA and HLLE under their reference names (defines/
method_names.hpp); neighbors method: brute only; eigen methods: arpack (the GPU
eigensolver) and dense. Errors print the tool's message and return 1.
"""
from __future__ import annotations

import argparse
import sys
import time

import numpy as np

from . import io as tkio

# defines/method_names.hpp:17-24 (the local-neighbourhood methods)
_METHODS = {
    "locally_linear_embedding": "lle", "lle": "lle",
    "local_tangent_space_alignment": "ltsa", "ltsa": "ltsa",
    "hessian_locally_linear_embedding": "hlle", "hlle": "hlle",
}
_NEIGHBORS = {"brute": "brute", "brute_force": "brute"}
_EIGEN = {"arpack": "arpack", "dense": "dense"}


def _error(msg: str) -> int:
    sys.stderr.write(f"[ERROR] {msg}\n")
    return 1


def _info(enabled: bool, msg: str) -> None:
    if enabled:
        sys.stderr.write(f"[INFO] {msg}\n")


def parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(prog="tapkee_gb300", description="Tapkee: a tool for dimensionality reduction.")
    p.add_argument("-i", "--input-file", default="/dev/stdin")
    p.add_argument("--transpose-input", action="store_true")
    p.add_argument("--transpose-output", action="store_true")
    p.add_argument("-o", "--output-file", default="/dev/stdout")
    p.add_argument("-d", "--delimiter", default=",")
    p.add_argument("--benchmark", action="store_true")
    p.add_argument("--verbose", action="store_true")
    p.add_argument("-m", "--method", default="locally_linear_embedding")
    p.add_argument("-nm", "--neighbors-method", default="brute")
    p.add_argument("-em", "--eigen-method", default="arpack")
    p.add_argument("-td", "--target-dimension", type=int, default=2)
    p.add_argument("-k", "--num-neighbors", type=int, default=10)
    p.add_argument("--eigenshift", type=float, default=1e-9)
    return p


def main(argv=None) -> int:
    a = parser().parse_args(argv)
    method = _METHODS.get(a.method)
    if method is None:
        return _error(f"Unknown method {a.method}")
    if a.neighbors_method not in _NEIGHBORS:
        if a.neighbors_method in ("vptree", "covertree"):
            return _error(f"Neighbors method {a.neighbors_method} is not provided by this library (brute only)")
        return _error(f"Unknown neighbors method {a.neighbors_method}")
    if a.eigen_method not in _EIGEN:
        if a.eigen_method == "randomized":
            return _error("Eigendecomposition method randomized is not provided by this library (arpack, dense)")
        return _error(f"Unknown eigendecomposition method {a.eigen_method}")
    if a.target_dimension <= 0:
        return _error("\"Only\" a positive target dimensionality larger than zero is possible in current "
                      "circumstances. Please visit other universe")
    if a.num_neighbors < 3:
        return _error("The provided number of neighbors is too small, consider at least 3.")
    data = tkio.read_data(a.input_file, a.delimiter)
    X = tkio.as_points(data, transposed=a.transpose_input)
    _info(a.verbose, f"Data contains {X.shape[0]} feature vectors with dimension of {X.shape[1]}")
    from . import api
    t0 = time.perf_counter()
    try:
        E = api.embed(np.ascontiguousarray(X.T), method=method, neighbors_method="brute",
                      eigen_method=_EIGEN[a.eigen_method], num_neighbors=a.num_neighbors,
                      target_dimension=a.target_dimension, nullspace_shift=a.eigenshift, check_connectivity=True)
    except api.TapkeeError as e:
        return _error(str(e))
    if a.benchmark:
        sys.stderr.write(f"[BENCHMARK] Embedding took {time.perf_counter() - t0:.6f} seconds\n")
    tkio.write_matrix(a.output_file, tkio.from_embedding(np.asarray(E), transposed=a.transpose_output), a.delimiter)
    return 0


if __name__ == "__main__":
    sys.exit(main())
