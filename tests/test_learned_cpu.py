"""Warm-start network host logic without a GPU: parameter layout and the weights file."""
from __future__ import annotations

import pytest


def test_parameter_layout():
    from iane_gb300.learned import LAYERS, WarmStartNet

    net = WarmStartNet("cpu", seed=0)
    n = 0
    for name, ci, co, _ in LAYERS:
        assert net.offsets[name] == (n, n + co * ci * 27)
        n += co * ci * 27 + co
    assert net.size == n == net.master.numel()
    assert 300_000 < n < 600_000


def test_weights_file_round_trip(tmp_path):
    import torch

    from iane_gb300.learned import WarmStartNet

    net = WarmStartNet("cpu", seed=4)
    path = tmp_path / "w.bin"
    net.save(path)
    other = WarmStartNet("cpu", seed=5)
    assert not torch.equal(other.master, net.master)
    other.load(path)
    assert torch.equal(other.master, net.master)
    assert torch.equal(other.p16, net.master.to(torch.bfloat16))
    raw = bytearray(path.read_bytes())
    raw[0] ^= 0xFF
    path.write_bytes(bytes(raw))
    with pytest.raises(ValueError):
        other.load(path)
    path.write_bytes(bytes(path.read_bytes()[:100]))
    with pytest.raises(ValueError):
        other.load(path)
