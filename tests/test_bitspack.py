"""Byte/bit layout of configurations: the reference's round-trip cases and its packed bytes."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import golden
from qmb_gb300 import bitspack


@pytest.mark.parametrize("size,hi", [(1, 2), (2, 4), (4, 16), (8, 256)])
@pytest.mark.parametrize("last", [16, 15, 14, 1000])
def test_pack_matches_reference_bytes(size, hi, last):
    g = golden("bitspack")
    x = torch.from_numpy(g[f"in_{size}_{last}"])
    packed = bitspack.pack_int(x, size)
    assert np.array_equal(packed.numpy(), g[f"packed_{size}_{last}"])
    assert torch.equal(bitspack.unpack_int(packed, size, last), x)


@pytest.mark.parametrize("size", [1, 2, 4, 8])
def test_round_trip_random(size):
    gen = torch.Generator().manual_seed(size)
    x = torch.randint(0, 1 << size, (7, 1000), generator=gen, dtype=torch.uint8)
    assert torch.equal(bitspack.unpack_int(bitspack.pack_int(x, size), size, 1000), x)


def test_site_layout():
    bits = torch.zeros(1, 20, dtype=torch.uint8)
    bits[0, 11] = 1
    packed = bitspack.pack_int(bits, 1)
    assert packed.tolist() == [[0, 1 << 3, 0]]


def test_multi_dimensional_and_empty():
    x = torch.tensor([[1, 0, 1, 1], [0, 0, 1, 0], [1, 1, 0, 1], [1, 0, 0, 1]], dtype=torch.uint8)
    assert torch.equal(bitspack.unpack_int(bitspack.pack_int(x, 1), 1, 4), x)
    e = torch.zeros(0, 9, dtype=torch.uint8)
    assert bitspack.pack_int(e, 1).shape == (0, 2)
