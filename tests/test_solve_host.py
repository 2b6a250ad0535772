"""Host logic of the batched solver: how the columns are split into blocks
(no GPU: the device memory queries are replaced)."""
from types import SimpleNamespace

import pytest
import torch

from fluxpy_gb300 import solve


@pytest.fixture
def free_memory(monkeypatch):
    state = {"free": 200 << 30}
    monkeypatch.setattr(torch.cuda, "mem_get_info", lambda *a: (state["free"], 280 << 30))
    monkeypatch.setattr(torch.cuda, "memory_reserved", lambda *a: 0)
    monkeypatch.setattr(torch.cuda, "memory_allocated", lambda *a: 0)
    return state


def _blocks(K, c):
    return [min(c, K - c0) for c0 in range(0, K, c)]


def test_column_blocks(free_memory):
    FF = SimpleNamespace(_num_zrows=1000)
    N = 2000
    # everything fits: one block of all columns, whatever K is
    for K in (1, 3, 8, 21, 1024, 8192):
        assert solve._auto_chunk(FF, N, K, False) == max(K, 8)
    # more than one block holds: equal blocks, multiples of 8, at most 8,192
    for K, c in ((8200, 4104), (16384, 8192), (16385, 5464), (50000, 7144)):
        got = solve._auto_chunk(FF, N, K, False)
        assert got == c and got % 8 == 0 and got <= solve._MAX_BLOCK_COLUMNS
        bl = _blocks(K, got)
        assert sum(bl) == K and max(bl) - min(bl) < 8 * len(bl)


def test_column_blocks_follow_free_memory(free_memory):
    N, zrows = 522242, 6952884
    FF = SimpleNamespace(_num_zrows=zrows)
    per_col = N * (7 * 4 + 2 * 2) + zrows * 4
    for free_gib in (8, 20, 40, 120):
        free_memory["free"] = free_gib << 30
        c = solve._auto_chunk(FF, N, 1024, False)
        assert c % 8 == 0 and 8 <= c <= 1024
        if c < 1024:
            # the blocks use at most 85 % of what is free after the reserve
            assert c * per_col <= 0.85 * ((free_gib - 6) << 30) + 8 * per_col
            assert len(_blocks(1024, c)) == -(-1024 // c)
    # nothing free: blocks of 8 columns, never fewer
    free_memory["free"] = 1 << 30
    assert solve._auto_chunk(FF, N, 1024, False) == 8
