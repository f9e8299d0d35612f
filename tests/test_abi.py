"""C ABI checks that need no GPU: the library loads, exports every entry point declared in
include/mtgpu.h, and its host-side table generator reproduces the reference's tables bit-exactly."""
import ctypes
import os
import re

import numpy as np
import pytest

from moltwister_gb300 import engine as E
from moltwister_gb300.build import build
from tests import golden_cases as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build()
    return E.load_library()


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(mtg_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert "mtg_create" in names and "mtg_run" in names
    for n in names:
        assert hasattr(lib, n), n


def test_version(lib):
    assert lib.mtg_version() == 1


def test_create_without_gpu_fails_cleanly(lib):
    """On a machine without a GPU, mtg_create must fail with an error code, never crash or fall
    back to a CPU path."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from moltwister_gb300 import workloads as W
    s, c = W.argon(ncell=2)
    with pytest.raises(E.MTGError) as ei:
        E.Engine(s, c)
    assert ei.value.code in (-1, -2)


@pytest.mark.parametrize("name", G.names())
def test_host_tables_bit_exact(lib, name):
    s, cfg, d = G.load(name)
    T = len(s.type_names())
    from oracle.oracle import reference_nb_layout
    ref_nb = reference_nb_layout(d["nb_table"], T)
    _, terms = s.nonbonded_pair_terms()
    rc = np.float32(cfg.cutoffradius)
    for pr in range(T * T):
        for ff, t in enumerate(terms[pr]):
            tab = E.term_profile(t, np.float32(0.01), rc)
            assert np.array_equal(tab.view(np.uint32), ref_nb[pr * 5 + ff].view(np.uint32))
    two_pi = np.float32(2.0 * np.pi)
    for i, t in enumerate(s.bond_terms):
        tab = E.term_profile(t, np.float32(0.01), rc)
        assert np.array_equal(tab.view(np.uint32), d["bond_table"].reshape(-1, 1000, 3)[i].view(np.uint32))
    for i, t in enumerate(s.angle_terms):
        tab = E.term_profile(t, np.float32(0.0), two_pi)
        assert np.array_equal(tab.view(np.uint32), d["angle_table"].reshape(-1, 1000, 3)[i].view(np.uint32))
    for i, t in enumerate(s.dihedral_terms):
        tab = E.term_profile(t, np.float32(0.0), two_pi)
        assert np.array_equal(tab.view(np.uint32), d["dih_table"].reshape(-1, 1000, 3)[i].view(np.uint32))
