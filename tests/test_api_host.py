"""Host-side refusals of the Python entry points (CPU, no GPU calls)."""
import numpy as np
import pytest

import tapkee_gb300 as tk
from tapkee_gb300 import api


def test_dense_eigensolver_refuses_large_n():
    """The dense path would hold an N x N FP64 matrix (320 GB at N = 200000): it is
    refused with the reference's wrong_parameter_error before anything is allocated."""
    n = api.DENSE_EIGEN_MAX_N + 1
    op = api.LocalOperator(idx=None, weights=None, row_ptr=np.zeros(n + 1, np.int64),
                           col_idx=np.zeros(0, np.int32), vals=np.zeros(0), k=8, method=0, target_dimension=2,
                           connectivity_retries=0, rows_uncertified=0)
    with pytest.raises(tk.WrongParameterError, match="dense eigensolver"):
        api.smallest_eigenvectors(op, 2, 1, eigen_method="dense")
    # the GPU path does not apply to td + skip > 14 either, so that also reaches the refusal
    with pytest.raises(tk.WrongParameterError, match="dense eigensolver"):
        api.smallest_eigenvectors(op, 14, 1, eigen_method="arpack")
