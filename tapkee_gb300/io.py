"""Delimiter-separated matrix files in the reference command-line tool's format.

read_data mirrors read_data (src/cli/util.hpp:73-116): one line per row, fields
split at a one-character delimiter, each field parsed as a real number with
fields that do not parse skipped; empty lines ignored; every row must have as
many values as the first ("Wrong data at line i" otherwise). write_matrix
mirrors write_matrix (src/cli/util.hpp:118-130): one row per line, values
written like a default C++ stream (6 significant digits), separated by the
delimiter. The tool reads a line as one vector to embed and transposes into the
library's features x samples layout unless told the file is already transposed
(src/cli/main.cpp:453-458); as_points / from_embedding do the same here for the
points-major arrays that tapkee_gb300 takes and returns.
"""
from __future__ import annotations

import re

import numpy as np

# what `istream >> double` (libstdc++ num_get) accepts at the start of a field:
# leading blanks, then a decimal number; the rest of the field is ignored. It
# reads neither "inf" / "nan" nor hexadecimal floats, so such fields are skipped.
_NUMBER = re.compile(r"\s*([+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)")


def _parse_field(field: str):
    m = _NUMBER.match(field)
    return float(m.group(1)) if m else None


def read_data(path: str, delimiter: str = ",") -> np.ndarray:
    """The file as a rows x columns float64 matrix (0 x 0 when it has no rows)."""
    if len(delimiter) < 1:
        raise ValueError("delimiter must be one character")
    d = delimiter[0]
    rows = []
    with open(path, "r") as f:
        for line in f:
            line = line.rstrip("\n")
            if not line:
                continue
            vals = []
            for field in line.split(d):
                v = _parse_field(field)
                if v is not None:
                    vals.append(v)
            rows.append(vals)
    if not rows:
        return np.zeros((0, 0))
    cols = len(rows[0])
    for i, r in enumerate(rows):
        if len(r) != cols:
            raise ValueError(f"Wrong data at line {i}")
    return np.array(rows, dtype=np.float64).reshape(len(rows), cols)


def _fmt(v: float) -> str:
    # a default-formatted C++ stream: %g with 6 significant digits, inf / nan
    if np.isnan(v):
        return "nan" if not np.signbit(v) else "-nan"
    if np.isinf(v):
        return "inf" if v > 0 else "-inf"
    return "%g" % v


def write_matrix(path: str, matrix, delimiter: str = ",") -> None:
    """Writes a 2-D matrix one row per line."""
    m = np.asarray(matrix, dtype=np.float64)
    if m.ndim != 2:
        raise ValueError("matrix must be 2-D")
    d = delimiter[0]
    with open(path, "w") as f:
        for row in m:
            f.write(d.join(_fmt(float(v)) for v in row))
            f.write("\n")


def as_points(matrix: np.ndarray, transposed: bool = False) -> np.ndarray:
    """Points-major N x D data from a file matrix: a line is a point unless the
    file holds one feature per line (transposed)."""
    return np.ascontiguousarray(matrix.T if transposed else matrix)


def from_embedding(embedding: np.ndarray, transposed: bool = False) -> np.ndarray:
    """The matrix the tool writes: one embedded point per line unless transposed."""
    return np.ascontiguousarray(embedding.T if transposed else embedding)
