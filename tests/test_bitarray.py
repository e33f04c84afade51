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
