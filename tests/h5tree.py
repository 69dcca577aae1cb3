"""Comparison of two parsed HDF5 trees (fortnet_gb300.hdf5lite nodes): the same groups,
datasets (dtype, shape, values) and attributes (type and value)."""

import numpy as np


def assert_same_tree(a, b, path=""):
    assert a.is_group == b.is_group, path
    assert set(a.attrs) == set(b.attrs), (path, set(a.attrs) ^ set(b.attrs))
    for k in a.attrs:
        x, y = a.attrs[k], b.attrs[k]
        if isinstance(x, str) or isinstance(y, str):
            assert x == y, (path, k, x, y)
        else:
            x, y = np.asarray(x), np.asarray(y)
            assert x.dtype == y.dtype and np.array_equal(x, y), (path, k, x, y)
    assert set(a.children) == set(b.children), (path, set(a.children) ^ set(b.children))
    for k in a.children:
        ca, cb = a.children[k], b.children[k]
        if ca.is_group:
            assert_same_tree(ca, cb, f"{path}/{k}")
        else:
            va, vb = ca.value, cb.value
            assert va.dtype == vb.dtype and va.shape == vb.shape, (path, k, va.shape, vb.shape)
            assert np.array_equal(va, vb), (path, k)
            assert set(ca.attrs) == set(cb.attrs), (path, k)
