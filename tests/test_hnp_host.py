"""Host logic of the heu.numpy-style layer (no GPU): plaintext conversion
and the broadcasting index maps used by element-wise ops
(numpy/evaluator.cc:160-185 casts shapes the NumPy way)."""

import numpy as np
import pytest

from heu_gb300 import hnp


def test_plaintext_arrays_keep_int64_and_big_values():
    a = hnp.PlaintextArray([[1, 2, 3], [4, 5, 6]])
    assert a.values.dtype == np.int64 and a.shape == (2, 3)
    assert str(a) == "[[1 2 3]\n [4 5 6]]"
    b = hnp.PlaintextArray([2 ** 70, -5])
    assert b.values.dtype == object and b.values.tolist() == [2 ** 70, -5]
    c = hnp.PlaintextArray(np.array([7, -7], dtype=object))
    assert c.values.dtype == np.int64
    assert a[1].to_numpy().tolist() == [4, 5, 6]


def test_broadcast_index_maps():
    shape, ix, iy = hnp._broadcast_index((2, 3), (3,))
    assert shape == (2, 3)
    assert ix.tolist() == [0, 1, 2, 3, 4, 5] and iy.tolist() == [0, 1, 2, 0, 1, 2]
    shape, ix, iy = hnp._broadcast_index((2, 1), (1, 3))
    assert shape == (2, 3) and ix.tolist() == [0, 0, 0, 1, 1, 1] and iy.tolist() == [0, 1, 2, 0, 1, 2]
    shape, ix, iy = hnp._broadcast_index((), (4,))
    assert shape == (4,) and ix.tolist() == [0, 0, 0, 0]
    with pytest.raises(ValueError, match="broadcast"):
        hnp._broadcast_index((2, 3), (2,))
