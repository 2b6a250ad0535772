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


def test_early_copy_ordering(monkeypatch):
    """The side-stream copy of candidate solutions (no GPU: streams and
    events are replaced by a log).  Each offer gathers B into facet order on
    the solver's stream, the side stream waits for that before it copies,
    the solver's stream waits for the copy before the gathered buffer is
    released or B changes, and only the offer of the final B is returned."""
    import contextlib

    log = []

    class Event:
        count = 0

        def __init__(self):
            Event.count += 1
            self.id = Event.count

        def record(self, s):
            log.append(("record", s.name, self.id))

        def synchronize(self):
            log.append(("sync", self.id))

    class Stream:
        def __init__(self, name="side"):
            self.name = name

        def wait_event(self, ev):
            log.append(("wait", self.name, ev.id))

    main = Stream("main")
    cur = [main]

    @contextlib.contextmanager
    def on(s):
        prev, cur[0] = cur[0], s
        try:
            yield
        finally:
            cur[0] = prev

    monkeypatch.setattr(torch.cuda, "Stream", lambda *a, **k: Stream("side"))
    monkeypatch.setattr(torch.cuda, "Event", Event)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a: cur[0])
    monkeypatch.setattr(torch.cuda, "stream", on)
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    monkeypatch.setattr(solve, "_COPY_STREAMS", {})
    perm = torch.tensor([2, 0, 1, 3])

    class Operator:
        def unpermute(self, xp):
            log.append(("gather", cur[0].name))
            return xp.index_select(0, perm)

    dst = torch.full((4, 2), float("nan"))
    ec = solve._EarlyCopy(Operator(), dst)
    B = torch.arange(8.0).reshape(4, 2)
    ec.offer(B)
    assert torch.equal(dst, B.index_select(0, perm)) and ec.copies == 1
    # gathered on the solver's stream; the side stream waits for it, then
    # records the end of its copy
    assert log == [("gather", "main"), ("record", "main", 1), ("wait", "side", 1),
                   ("record", "side", 2)]
    # the solver changes B: its stream waits for the copy first
    log.clear()
    ec.fence()
    assert log == [("wait", "main", 2)]
    B += 1
    ec.offer(B)
    ec.offer(B)       # a second offer waits for the first copy before the gather
    assert log[1:3] == [("gather", "main"), ("record", "main", 3)]
    i = log.index(("record", "side", 4))
    assert log[i + 1:i + 3] == [("wait", "main", 4), ("gather", "main")]
    assert ec.copies == 3
    # a check that accepts another tensor gets nothing back; the copy in
    # flight is waited for
    log.clear()
    assert ec.result(B.clone()) is None and log == [("wait", "main", 6)]
    # the accepted B: the host waits for its copy and gets the gathered B
    ec.offer(B)
    log.clear()
    Bu = ec.result(B)
    assert log == [("sync", 8), ("wait", "main", 8)]
    assert torch.equal(Bu, B.index_select(0, perm)) and torch.equal(dst, Bu)


def test_argument_checks_before_device_use():
    """The reference's argument errors (compressed_form_factors.py:737-738,
    879-885; solve.py:9-22) come before any device work."""
    import numpy as np
    from fluxpy_gb300.compressed_form_factors import (CompressedFormFactorMatrix,
                                                      CompressedKernelMatrix)
    with pytest.raises(RuntimeError, match="tol should be a nonnegative float"):
        CompressedFormFactorMatrix(None, tol=-1e-5)
    with pytest.raises(RuntimeError, match="invalid max_depth type"):
        CompressedFormFactorMatrix(None, max_depth=2.0)
    with pytest.raises(RuntimeError, match="invalid max_depth value"):
        CompressedFormFactorMatrix(None, max_depth=0)
    with pytest.raises(RuntimeError, match="max_depth not specified"):
        CompressedFormFactorMatrix(None, force_max_depth=True)
    with pytest.raises(ValueError, match="need 0 < rho <= 1"):
        CompressedKernelMatrix(None, 0.0)
    with pytest.raises(ValueError, match="need 0 < rho <= 1"):
        CompressedKernelMatrix(None, 1.5)
    with pytest.raises(ValueError, match='albedo_placement must be "left" or "right"'):
        CompressedKernelMatrix(None, 0.5, "middle")
    E = np.ones(4)
    with pytest.raises(Exception, match='albedo_placement must be "left" or "right"'):
        solve.solve_radiosity(None, E, 0.12, "middle")
    with pytest.raises(ValueError, match="batched methods only"):
        solve.solve_radiosity(None, E, 0.12, out=np.empty(4))
    with pytest.raises(ValueError, match="right albedo placement"):
        solve.solve_radiosity(None, E[:, None], 0.12, "left", method="batched-bf16")
