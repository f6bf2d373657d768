"""Bit packing of small unsigned integers into bytes (API of qmb/bitspack.py:8-94).

Configurations reach the engine packed by ``pack_int(bits, 1)``: element e of
the last dimension lands in byte e // 8 at bit e % 8, least significant bit
first, and the last byte is zero-padded.  The engine's kernels rely on exactly
this layout: they read a row as big-endian 64-bit key words (row byte b in
word b // 8 at bits (7 - b % 8) * 8 .. +7), so that comparing words as
unsigned integers is the reference's lexicographic byte order, and site s
sits in word s // 64 at bit (7 - (s // 8) % 8) * 8 + s % 8.
"""

from __future__ import annotations

import torch

__all__ = ["pack_int", "unpack_int"]


def pack_int(tensor: torch.Tensor, size: int) -> torch.Tensor:
    """Pack the last dimension of a uint8 tensor, ``size`` bits per element (1, 2, 4 or 8)."""
    if tensor.dtype != torch.uint8:
        raise TypeError("pack_int expects a uint8 tensor")
    if size not in (1, 2, 4, 8):
        raise ValueError("size must be 1, 2, 4 or 8")
    per_byte = 8 // size
    last = tensor.shape[-1]
    padded = -(-last // per_byte) * per_byte
    if padded != last:
        tensor = torch.nn.functional.pad(tensor, (0, padded - last))
    groups = tensor.reshape(*tensor.shape[:-1], padded // per_byte, per_byte)
    shifts = torch.arange(0, 8, size, device=tensor.device, dtype=torch.uint8)
    mask = (1 << size) - 1
    return torch.bitwise_left_shift(torch.bitwise_and(groups, mask), shifts).sum(dim=-1, dtype=torch.uint8)


def unpack_int(tensor: torch.Tensor, size: int, last_dim: int) -> torch.Tensor:
    """Inverse of ``pack_int``: ``last_dim`` elements of ``size`` bits from each packed row."""
    if tensor.dtype != torch.uint8:
        raise TypeError("unpack_int expects a uint8 tensor")
    if size not in (1, 2, 4, 8):
        raise ValueError("size must be 1, 2, 4 or 8")
    shifts = torch.arange(0, 8, size, device=tensor.device, dtype=torch.uint8)
    mask = (1 << size) - 1
    fields = torch.bitwise_and(torch.bitwise_right_shift(tensor.unsqueeze(-1), shifts), mask)
    return fields.reshape(*tensor.shape[:-1], tensor.shape[-1] * (8 // size))[..., :last_dim]
