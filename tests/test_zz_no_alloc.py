"""mtg_neighbors_noalloc: the context-free, no-allocation neighbour list.

It must give exactly what the context entry point mtg_get_neighbors gives (which the parity
tests pin bit-exactly to the reference's lists), on two calls in a row, because its working
arrays live in one device array that every call reuses.  Collected last on purpose: it must pass
both alone and after every other test has used the device.
"""
import numpy as np
import pytest

from moltwister_gb300 import engine as E
from tests import golden_cases as G


@pytest.fixture(scope="module")
def lib():
    from moltwister_gb300.build import build
    build()
    return E.load_library()


def test_rejects_oversize_before_touching_the_device(lib):
    # 500 atoms in a 2000 A box with a 1 A cutoff: 2000^3 cells, far beyond the scratch array.
    r = np.zeros((500, 3))
    cnt = np.zeros(500, np.int32)
    with pytest.raises(E.MTGError) as ei:
        E.neighbors_noalloc(r.ctypes.data, 500, (2000.0, 2000.0, 2000.0), 1.0, 0.0, 0, cnt.ctypes.data, 0)
    assert ei.value.code == E.MTG_E_INVALID
    assert "scratch" in str(ei.value)


def _context_lists(name):
    s, cfg, _ = G.load(name)
    cnt, lst = E.Engine(s, cfg).neighbors()
    return s, cfg, cnt, lst


@pytest.mark.gpu
@pytest.mark.parametrize("name", G.names())
def test_matches_context_entry_point_twice(lib, name):
    import torch
    s, cfg, cnt_ref, lst_ref = _context_lists(name)
    dev = torch.device("cuda:0")
    r = torch.tensor(np.ascontiguousarray(s.r, np.float64), device=dev)
    m = int(cnt_ref.max())
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        cnt = torch.full((s.n,), -7, dtype=torch.int32, device=dev)
        lst = torch.full((s.n, m), -7, dtype=torch.int32, device=dev)
        need = E.neighbors_noalloc(r.data_ptr(), s.n, s.box, cfg.cutoffradius, cfg.neighshell, m,
                                   cnt.data_ptr(), lst.data_ptr(), stream)
        assert need == 0, call
        c = cnt.cpu().numpy()
        L = lst.cpu().numpy()
        assert np.array_equal(c, cnt_ref), call
        for k in range(s.n):
            assert np.array_equal(L[k, :c[k]], lst_ref[k, :c[k]]), (call, k)


@pytest.mark.gpu
def test_truncation_then_full_capacity(lib):
    """A call that truncates (sets the overflow flag in the scratch) followed by one that fits:
    the second must report 0, i.e. the flag is cleared at the start of every call."""
    import torch
    s, cfg, cnt_ref, lst_ref = _context_lists("water648_nvt")
    dev = torch.device("cuda:0")
    r = torch.tensor(np.ascontiguousarray(s.r, np.float64), device=dev)
    m = int(cnt_ref.max())
    short = m // 2
    cnt = torch.zeros(s.n, dtype=torch.int32, device=dev)
    lst = torch.zeros((s.n, short), dtype=torch.int32, device=dev)
    need = E.neighbors_noalloc(r.data_ptr(), s.n, s.box, cfg.cutoffradius, cfg.neighshell, short,
                               cnt.data_ptr(), lst.data_ptr())
    assert need == m
    c = cnt.cpu().numpy()
    L = lst.cpu().numpy()
    assert np.array_equal(c, cnt_ref)                   # full counts even when truncated
    for k in range(s.n):
        kk = min(c[k], short)
        assert np.array_equal(L[k, :kk], lst_ref[k, :kk])
    lst = torch.zeros((s.n, m), dtype=torch.int32, device=dev)
    assert E.neighbors_noalloc(r.data_ptr(), s.n, s.box, cfg.cutoffradius, cfg.neighshell, m,
                               cnt.data_ptr(), lst.data_ptr()) == 0


@pytest.mark.gpu
def test_rejects_host_pointers(lib):
    import torch
    torch.cuda.init()
    s, cfg, _ = G.load("argon500_nvt")
    r = np.ascontiguousarray(s.r, np.float64)
    cnt = torch.zeros(s.n, dtype=torch.int32, device="cuda:0")
    with pytest.raises(E.MTGError) as ei:
        E.neighbors_noalloc(r.ctypes.data, s.n, s.box, cfg.cutoffradius, cfg.neighshell, 0, cnt.data_ptr(), 0)
    assert ei.value.code == E.MTG_E_INVALID
