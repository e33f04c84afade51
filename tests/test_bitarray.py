"""The device bit sets of the Python mirror (BitArray, ngsxfem_gb300/xfem.py)
on the CPU: packing a bool tensor (from_bool, which the dof marking of
GetDofsOfElements uses) agrees with the numpy packing and unpacks back
(bool_tensor), including bit 63 of a word and a ragged last word."""
import numpy as np
import torch

import ngsxfem_gb300.xfem as X


def test_pack_unpack_round_trip(monkeypatch):
    monkeypatch.setattr(X, "_dev", lambda: "cpu")  # host logic only: the library itself needs a GPU
    rng = np.random.default_rng(1)
    for n in (1, 63, 64, 65, 200, 1000):
        bits = rng.random(n) < 0.4
        bits[min(63, n - 1)] = True
        a = X.BitArray.from_bool(torch.from_numpy(bits))
        b = X.BitArray.from_numpy(bits)
        assert a.n == b.n == n
        assert torch.equal(a.words.cpu(), b.words.cpu())
        assert np.array_equal(a.bool_tensor().cpu().numpy(), bits)
        assert np.array_equal(a.numpy(), bits)


def test_restrict_takes_spatial_spaces_only():
    """Restrict / Compress views share the space's handle; space-time spaces
    (their own lifetime) and tensor-mesh H1 (no handle) are refused."""
    import pytest

    st = object.__new__(X.SpaceTimeFESpace)
    with pytest.raises(NotImplementedError):
        X.Restrict(st, None)
    quad = object.__new__(X.H1)
    quad.h = None
    with pytest.raises(NotImplementedError):
        X.Compress(quad, None)
