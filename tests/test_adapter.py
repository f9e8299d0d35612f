"""The drop-in adapter (oracle/ref/adapter.cpp) against the Python binding.

The adapter builds mtg_system_desc / mtg_config_desc from MolTwister's own objects (CMDFFMatrices,
the MDFF lists, CMolTwisterStateTools) the way the MolTwister host build would; `mtref desc` runs
it inside the reference build.  For every golden case the descriptor must equal what the Python
binding (moltwister_gb300.engine.system_desc / config_desc) passes for the same system: atoms,
types, molecule indices, topology and the reference's tables bit for bit, term kinds exactly and
term parameters to the digits the MDFF classes print them with (getArguments: 6 to 10 decimals).
Needs the reference build (oracle/_ref/mtref); skipped where it is absent."""
import os
import tempfile

import numpy as np
import pytest

from tests import golden_cases as G

HARNESS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle", "_ref", "mtref")
CASES = [n for n in G.names() if n not in ("argon4000_nvt", "water9000_ref")]

pytestmark = pytest.mark.skipif(not os.path.exists(HARNESS), reason="reference build (oracle/_ref/mtref) absent")


def adapter_desc(s, cfg):
    from oracle.mtb import read_mtb
    from oracle.sysfile import run_harness
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "d.mtb")
        run_harness(["desc", out], s, cfg)
        return read_mtb(out)


def binding_arrays(s, cfg):
    import ctypes as C
    from moltwister_gb300.engine import MAXFF, NPTS, config_desc, system_desc
    keep = []
    sd = system_desc(s, keep)
    T, n = sd.n_types, sd.n_atoms

    def arr(ptr, count, ctype):
        if not ptr or count == 0:
            return np.zeros(0)
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(count,)).copy()

    def terms(ptr, count):
        if not ptr or count == 0:
            return np.zeros(0, np.int32), np.zeros((0, 4))
        from moltwister_gb300.engine import Term
        tp = C.cast(ptr, C.POINTER(Term))
        return np.array([tp[k].kind for k in range(count)], np.int32), np.array([list(tp[k].p) for k in range(count)])

    nk, npar = terms(sd.nb_terms, T * T * MAXFF)
    bk, bp = terms(sd.bond_terms, sd.n_bond_types)
    ak, ap = terms(sd.angle_terms, sd.n_angle_types)
    dk, dp = terms(sd.dih_terms, sd.n_dih_types)
    return dict(n=n, T=T, r=arr(sd.r, 3 * n, C.c_double), mass=arr(sd.mass, n, C.c_double),
                charge=arr(sd.charge, n, C.c_double), type=arr(sd.type, n, C.c_int32), mol=arr(sd.mol, n, C.c_int32),
                mobile=arr(sd.mobile, n, C.c_uint8), box=np.array(sd.box[:]),
                nb_count=arr(sd.nb_count, T * T, C.c_int32), nb_kind=nk, nb_p=npar, bond_kind=bk, bond_p=bp,
                angle_kind=ak, angle_p=ap, dih_kind=dk, dih_p=dp,
                bonds=arr(sd.bonds, 3 * sd.n_bonds, C.c_int32), angles=arr(sd.angles, 4 * sd.n_angles, C.c_int32),
                dihedrals=arr(sd.dihedrals, 5 * sd.n_dihedrals, C.c_int32), cfg=config_desc(cfg))


@pytest.mark.parametrize("name", CASES)
def test_adapter_descriptor_matches_the_binding(name):
    from oracle.oracle import reference_nb_layout
    s, cfg, d = G.load(name)
    a = adapter_desc(s, cfg)
    b = binding_arrays(s, cfg)
    T = b["T"]
    for key in ("r", "mass", "charge", "box"):
        assert np.array_equal(a[key], b[key]), key
    for key in ("type", "mol", "mobile", "nb_count", "bonds", "angles", "dihedrals"):
        assert np.array_equal(a[key].astype(np.int64), b[key].astype(np.int64)), key
    for grp in ("nb", "bond", "angle", "dih"):
        assert np.array_equal(a[grp + "_kind"], b[grp + "_kind"]), grp
        pa, pb = a[grp + "_p"].reshape(-1, 4), b[grp + "_p"].reshape(-1, 4)
        assert np.allclose(pa, pb, rtol=1e-6, atol=1e-9), (grp, pa, pb)
    # the reference's own tables, reordered into the library's layout
    assert np.array_equal(a["nb_tables"].reshape(-1, 1000, 3).view(np.uint32),
                          reference_nb_layout(d["nb_table"], T).view(np.uint32))
    assert np.array_equal(a["bond_tables"].reshape(-1, 3).view(np.uint32), d["bond_table"].reshape(-1, 3).view(np.uint32))
    assert np.array_equal(a["angle_tables"].reshape(-1, 3).view(np.uint32), d["angle_table"].reshape(-1, 3).view(np.uint32))
    c = b["cfg"]
    want = [c.ensemble, c.temperature_nh_len, c.temperature_respa, c.pressure_nh_len, c.pressure_respa, c.timestep,
            c.temperature, c.temperature_relax, c.pressure, c.pressure_relax, c.cutoff_radius, c.neigh_shell,
            c.cutoff_force, c.scale12, c.scale13, c.scale14, c.scale1N]
    assert np.allclose(a["cfg"], want, rtol=1e-12), (a["cfg"], want)
