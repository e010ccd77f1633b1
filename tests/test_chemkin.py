"""CHEMKIN-format mechanism reader and writer (pelelm_gb300.mech.chemkin), CPU only.

The synthetic mechanisms are written out in CHEMKIN form and read back: stoichiometry, reaction
types, Arrhenius/LOW/TROE/efficiency data come back exactly (the writer prints them at full
double precision), thermo to the fixed format's nine significant digits, and the oracle's
production rates of the re-read mechanism match the original's. A small hand-written input
exercises each syntax feature (units, third-body efficiencies, (+M) and (+species) falloff,
TROE, REV, DUPLICATE, comments, coefficients) and the error paths."""
import numpy as np
import pytest

from pelelm_gb300.mech.chemkin import AVOGADRO, ChemkinError, read_chemkin, write_chemkin
from pelelm_gb300.mech.model import R_CAL
from pelelm_gb300.workloads import CONFIGS, load_mechanism, make_cells

MECHS = ["lidryer_syn", "drm19_syn", "gri_syn"]
CFG_OF = {"lidryer_syn": "lidryer_amr120", "drm19_syn": "drm19_2M", "gri_syn": "gri_1M"}


@pytest.mark.parametrize("name", MECHS)
@pytest.mark.parametrize("separate_thermo", [True, False])
def test_round_trip_of_the_synthetic_mechanisms(tmp_path, name, separate_thermo):
    m = load_mechanism(name)
    chem, therm = tmp_path / "chem.inp", tmp_path / "therm.dat"
    write_chemkin(m, str(chem), str(therm) if separate_thermo else None)
    r = read_chemkin(str(chem), str(therm) if separate_thermo else None, name=name, synthetic=True)
    assert r.elements == m.elements
    assert [s.name for s in r.species] == [s.name for s in m.species]
    for a, b in zip(r.species, m.species):
        assert a.composition == b.composition and a.Tmid == b.Tmid
        assert abs(a.W - b.W) <= 1e-12 * b.W
        np.testing.assert_allclose(a.low, b.low, rtol=6e-9, atol=0)
        np.testing.assert_allclose(a.high, b.high, rtol=6e-9, atol=0)
    assert len(r.reactions) == len(m.reactions)
    for a, b in zip(r.reactions, m.reactions):
        assert (a.kind, a.reactants, a.products, a.reversible) == (b.kind, b.reactants, b.products, b.reversible)
        assert a.rate == b.rate and a.low == b.low and a.troe == b.troe
        assert a.efficiencies == b.efficiencies and a.rev is None and not a.duplicate
    # the text is a fixed point: writing what was read gives the same file
    chem2 = tmp_path / "chem2.inp"
    therm2 = tmp_path / "therm2.dat"
    write_chemkin(r, str(chem2), str(therm2) if separate_thermo else None)
    assert chem2.read_text() == chem.read_text()
    if separate_thermo:
        assert therm2.read_text() == therm.read_text()


@pytest.mark.parametrize("name", MECHS)
def test_reread_mechanism_gives_the_same_rates(tmp_path, oracle_mod, name):
    """Production rates of the re-read mechanism (thermo at nine digits) against the original's,
    through the oracle, on workload states."""
    m = load_mechanism(name)
    write_chemkin(m, str(tmp_path / "chem.inp"), str(tmp_path / "therm.dat"))
    r = read_chemkin(str(tmp_path / "chem.inp"), str(tmp_path / "therm.dat"), name=name)
    r.to_flat(str(tmp_path / "r.mech"))
    m.to_flat(str(tmp_path / "m.mech"))
    cs = make_cells(CONFIGS[CFG_OF[name]], 64, seed=3)
    W = np.array([s.W for s in m.species])
    C = cs.rY / W[None, :]
    wa = oracle_mod.OracleMech(str(tmp_path / "m.mech")).wdot(cs.T, C)
    wb = oracle_mod.OracleMech(str(tmp_path / "r.mech")).wdot(cs.T, C)
    scale = np.abs(wa).max(axis=1, keepdims=True)
    assert np.max(np.abs(wb - wa) / scale) < 1e-6


CHEM = """! a made-up five-reaction test input (not a real mechanism)
ELEM H O N AR END
SPECIES
H2 O2 H O OH   ! radicals
H2O HO2 N2 AR
END
REACTIONS KJOULES/MOLE MOLECULES
H+O2 = O+OH            3.0E-10  0.0   70.0
H2 + O => H + OH       1.0E-11  1.5   30.0
2OH+M<=>H2O+O+M        1.0E-30 -1.0    0.0
   H2O/5.0/ AR/0.5/
H+O2(+M) = HO2(+M)     7.5E-11  0.6    0.0
   LOW / 1.0E-30 -1.5 0.0 /
   TROE / 0.5 100.0 2000.0 1.0E4 /
H+OH(+H2O)=H2O(+H2O)   2.0E-10  0.0    0.0
   LOW / 3.0E-29 -2.0 0.0/
HO2+H=H2+O2            1.0E-11  0.0    5.0
   DUPLICATE
HO2+H=H2+O2            2.0E-10  0.0   10.0
   REV / 1.0E-12 0.5 200.0 /
   DUP
END
"""

THERM = ["THERMO ALL", "   300.000  1000.000  5000.000"]


def _therm(name, comp, a_hi, a_lo, tmid=1000.0):
    field = "".join(f"{e:<2}{n:>3d}" for e, n in comp) + " " * (5 * (4 - len(comp)))
    l1 = f"{name:<18}{'':6}{field}G{300.0:10.3f}{5000.0:10.3f}{tmid:8.2f}"
    c = a_hi + a_lo
    return [f"{l1:<79}1",
            "".join(f"{v:15.8E}" for v in c[0:5]) + "    2",
            "".join(f"{v:15.8E}" for v in c[5:10]) + "    3",
            "".join(f"{v:15.8E}" for v in c[10:14]) + " " * 15 + "    4"]


def _write_inputs(tmp_path, chem=CHEM):
    # arbitrary smooth coefficient sets, enough for the parser (no physical meaning)
    comps = {"H2": [("H", 2)], "O2": [("O", 2)], "H": [("H", 1)], "O": [("O", 1)], "OH": [("O", 1), ("H", 1)],
             "H2O": [("H", 2), ("O", 1)], "HO2": [("H", 1), ("O", 2)], "N2": [("N", 2)], "AR": [("AR", 1)]}
    lines = list(THERM)
    for k, (s, comp) in enumerate(comps.items()):
        hi = [3.0 + 0.1 * k, 1e-3, -2e-7, 3e-11, -1e-15, -1000.0 * k, 2.0 + k]
        lo = [3.5 - 0.1 * k, -1e-3, 2e-6, -1e-9, 2e-13, -1100.0 * k, 1.0 + k]
        lines += _therm(s, comp, hi, lo)
    lines.append("END")
    (tmp_path / "chem.inp").write_text(chem)
    (tmp_path / "therm.dat").write_text("\n".join(lines) + "\n")
    return str(tmp_path / "chem.inp"), str(tmp_path / "therm.dat")


def test_parser_features_and_unit_conversion(tmp_path):
    chem, therm = _write_inputs(tmp_path)
    m = read_chemkin(chem, therm, name="t")
    assert m.elements == ["H", "O", "N", "Ar"]
    assert [s.name for s in m.species] == ["H2", "O2", "H", "O", "OH", "H2O", "HO2", "N2", "AR"]
    assert m.species[m.index("AR")].composition == {"Ar": 1}
    assert m.species[m.index("OH")].W == pytest.approx(15.999 + 1.008)
    r = m.reactions
    assert len(r) == 7
    ea = 70.0 * 1000.0 / 4.184
    assert r[0].kind == "elementary" and r[0].reversible and r[0].rate.Ea == pytest.approx(ea)
    assert r[0].rate.A == pytest.approx(3.0e-10 * AVOGADRO)          # bimolecular: x N_A
    assert not r[1].reversible and r[1].rate.beta == 1.5
    assert r[2].kind == "three_body" and r[2].reactants == {"OH": 2}
    assert r[2].rate.A == pytest.approx(1.0e-30 * AVOGADRO ** 2)      # +M: termolecular
    assert r[2].efficiencies == {"H2O": 5.0, "AR": 0.5}
    assert r[3].kind == "falloff" and r[3].troe == [0.5, 100.0, 2000.0, 1.0e4]
    assert r[3].rate.A == pytest.approx(7.5e-11 * AVOGADRO) and r[3].low.A == pytest.approx(1.0e-30 * AVOGADRO ** 2)
    assert r[4].kind == "falloff" and r[4].troe is None               # Lindemann, (+H2O) only
    assert r[4].efficiencies["H2O"] == 1.0 and r[4].efficiencies["N2"] == 0.0
    assert r[5].duplicate and r[6].duplicate
    assert r[6].rev is not None and r[6].rev.A == pytest.approx(1.0e-12 * AVOGADRO)
    assert r[6].rev.Ea == pytest.approx(200.0 * 1000.0 / 4.184)
    # REV is read and kept, but the rate kernels take reverse rates from K_c only
    with pytest.raises(ValueError, match="REV"):
        m.to_flat(str(tmp_path / "t.mech"))
    # KELVINS: E/R given directly
    chem2 = CHEM.replace("KJOULES/MOLE MOLECULES", "KELVINS")
    m2 = read_chemkin(*_write_inputs(tmp_path, chem2), name="t2")
    assert m2.reactions[0].rate.Ea == pytest.approx(70.0 * R_CAL) and m2.reactions[0].rate.A == 3.0e-10


@pytest.mark.parametrize("edit,msg", [
    (("H+O2 = O+OH", "H+O3 = O+OH"), "unknown species"),
    (("   DUPLICATE\n", ""), "DUPLICATE"),
    (("   TROE / 0.5 100.0 2000.0 1.0E4 /", "   SRI / 0.5 100.0 2000.0 /"), "SRI"),
    (("2OH+M<=>H2O+O+M        1.0E-30 -1.0    0.0", "2OH<=>H2O+O            1.0E-30 -1.0    0.0"),
     "efficiencies"),
    (("H2 + O => H + OH       1.0E-11  1.5   30.0", "H2 + O => H + OH       1.0E-11  1.5   30.0\n   LOW / 1 2 3 /"),
     "LOW"),
])
def test_parser_errors(tmp_path, edit, msg):
    chem = CHEM.replace(*edit)
    assert chem != CHEM
    with pytest.raises(ChemkinError, match=msg):
        read_chemkin(*_write_inputs(tmp_path, chem), name="bad")


def test_converted_mechanism_compiles_as_a_library_unit(tmp_path):
    """A mechanism read from CHEMKIN input becomes a library entry with no source edit: the
    build generates its kernel header, tables, unit and registry line from the JSON. Here the
    9-species mechanism, written out and read back under a new name, goes through the same
    generators and its unit compiles for sm_103a (nvcc cross-compiles on a host without GPU)."""
    import os
    import shutil
    import subprocess
    from pelelm_gb300 import _build
    from pelelm_gb300.mech import codegen
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    m = load_mechanism("lidryer_syn")
    write_chemkin(m, str(tmp_path / "chem.inp"), str(tmp_path / "therm.dat"))
    r = read_chemkin(str(tmp_path / "chem.inp"), str(tmp_path / "therm.dat"), name="lidryer_ck")
    gen = tmp_path / "gen"
    gen.mkdir()
    (gen / "mech_lidryer_ck.cuh").write_text(codegen.gen_header(r))
    (gen / "tab_lidryer_ck.cuh").write_text(codegen.gen_tables(r, "constant"))
    (gen / "tabg_lidryer_ck.cuh").write_text(codegen.gen_tables(r, "global"))
    unit = gen / "unit_lidryer_ck.cu"
    unit.write_text(f'#include "mech_lidryer_ck.cuh"\n#include "../reactor_registry.cuh"\n'
                    "namespace pgb_host {\n"
                    f"extern const MechEntry kEntry_lidryer_ck = PGB_MECH_ENTRY(pgb::Mech_lidryer_ck);\n}}\n")
    assert codegen.kernel_family(r) == "thread"
    csrc_gen = os.path.join(_build.CSRC, "gen")
    cmd = [nvcc, *_build.NVFLAGS, *_build.ARCH, "-I", csrc_gen, "-c", str(unit), "-o", str(tmp_path / "u.o")]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    assert "lidryer_ck" in subprocess.run(["nm", "-C", str(tmp_path / "u.o")], capture_output=True, text=True).stdout
