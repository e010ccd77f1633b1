"""Physical model used to build synthetic NASA-7 thermo for a species from its formula.

The real mechanism thermo files (PelePhysics ``Support/Mechanism/Models/*``) are not
available, so species thermo is *computed* here from textbook physics and a fixed seed:

* a valence skeleton (heavy atoms C/N chained, O attached to the least-saturated C/N,
  hydrogens filled in, leftover valence turned into multiple bonds, the rest unpaired
  electrons);
* heat of formation from average bond enthalpies and atomisation enthalpies,
  plus a seeded perturbation (elemental reference species are exactly 0);
* c_p(T) from a rigid-rotor / harmonic-oscillator model with seeded vibrational
  temperatures;
* S(298.15 K) from the Sackur-Tetrode, rigid-rotor, oscillator and electronic terms;
* a least-squares NASA-7 fit on [300, Tmid] and [Tmid, 3500] with h and s continuous at Tmid.

The NASA-7 form itself is the one in ``Docs/source/manual/Model.rst:271-296``.
"""
from __future__ import annotations

import math
import re
from typing import Dict, List, Tuple

import numpy as np

VALENCE = {"C": 4, "N": 3, "O": 2, "H": 1}
ATOM_DHF = {"H": 218.0, "C": 716.7, "N": 472.7, "O": 249.2, "Ar": 0.0}  # kJ/mol
# average bond enthalpies, kJ/mol, keyed by sorted pair and order
BOND_E = {
    ("H", "H", 1): 436.0, ("C", "H", 1): 413.0, ("H", "N", 1): 391.0, ("H", "O", 1): 463.0,
    ("C", "C", 1): 348.0, ("C", "C", 2): 614.0, ("C", "C", 3): 839.0,
    ("C", "N", 1): 293.0, ("C", "N", 2): 615.0, ("C", "N", 3): 891.0,
    ("C", "O", 1): 358.0, ("C", "O", 2): 745.0, ("C", "O", 3): 1072.0,
    ("N", "N", 1): 163.0, ("N", "N", 2): 418.0, ("N", "N", 3): 945.0,
    ("N", "O", 1): 201.0, ("N", "O", 2): 607.0,
    ("O", "O", 1): 146.0, ("O", "O", 2): 498.0,
}
ELEMENTAL_REFS = {"H2", "O2", "N2", "AR"}
KB = 1.380649e-16    # erg/K
HPL = 6.62607015e-27  # erg s
NA = 6.02214076e23
R_J = 8.31446261815324  # J/mol/K
P0 = 1.01325e6


def parse_formula(name: str) -> Dict[str, int]:
    """'CH2(S)' -> {'C':1,'H':2}; 'AR' -> {'Ar':1}."""
    if name.upper() == "AR":
        return {"Ar": 1}
    base = re.sub(r"\(.*\)$", "", name)
    comp: Dict[str, int] = {}
    for el, n in re.findall(r"([A-Z][a-z]?)(\d*)", base):
        if not el:
            continue
        comp[el] = comp.get(el, 0) + (int(n) if n else 1)
    return comp


def skeleton(comp: Dict[str, int]) -> Tuple[List[Tuple[str, str, int]], int]:
    """Return (bonds as (el_a, el_b, order), number of unpaired electrons)."""
    atoms = []
    for el in ("C", "N", "O"):
        atoms += [el] * comp.get(el, 0)
    nh = comp.get("H", 0)
    if "Ar" in comp:
        return [], 0
    if not atoms:  # only hydrogen
        if nh == 1:
            return [], 1
        return [("H", "H", 1)] * (nh // 2), nh % 2
    free = [VALENCE[a] for a in atoms]
    adj: Dict[Tuple[int, int], int] = {}
    cn = [i for i, a in enumerate(atoms) if a in ("C", "N")]
    oxy = [i for i, a in enumerate(atoms) if a == "O"]
    # C/N chain
    for a, b in zip(cn[:-1], cn[1:]):
        adj[(a, b)] = 1
        free[a] -= 1
        free[b] -= 1
    # oxygens: attach to the C/N with most free valence, else chain on previous O
    prev_o = None
    for o in oxy:
        if cn:
            host = max(cn, key=lambda i: (free[i], -i))
            if free[host] > 0:
                adj[(host, o)] = 1
                free[host] -= 1
                free[o] -= 1
                continue
        if prev_o is not None:
            adj[(prev_o, o)] = 1
            free[prev_o] -= 1
            free[o] -= 1
        prev_o = o
    bonds: List[Tuple[str, str, int]] = []
    # hydrogens: to heavy atom with most free valence (C first)
    for _ in range(nh):
        host = max(range(len(atoms)), key=lambda i: (free[i], atoms[i] == "C", -i))
        if free[host] <= 0:
            break
        free[host] -= 1
        bonds.append(tuple(sorted((atoms[host], "H"))) + (1,))
    # raise bond orders where both ends have free valence
    changed = True
    while changed:
        changed = False
        for (a, b), order in list(adj.items()):
            if free[a] > 0 and free[b] > 0 and order < 3:
                adj[(a, b)] = order + 1
                free[a] -= 1
                free[b] -= 1
                changed = True
    # carbon monoxide style: C=O with two free on C -> C#O
    for (a, b), order in list(adj.items()):
        pair = {atoms[a], atoms[b]}
        if pair == {"C", "O"} and order == 2 and len(atoms) == 2 and free[a] + free[b] == 2:
            adj[(a, b)] = 3
            free[a] = free[b] = 0
    for (a, b), order in adj.items():
        ea, eb = sorted((atoms[a], atoms[b]))
        bonds.append((ea, eb, min(order, 3 if (ea, eb, 3) in BOND_E else 2)))
    unpaired = sum(max(f, 0) for f in free)
    return bonds, unpaired


def bond_energy(b: Tuple[str, str, int]) -> float:
    key = b
    while key not in BOND_E and key[2] > 1:
        key = (key[0], key[1], key[2] - 1)
    return BOND_E[key]


def dhf_kj(name: str, comp: Dict[str, int], rng: np.random.Generator) -> float:
    if name.upper() in ELEMENTAL_REFS:
        return 0.0
    bonds, unpaired = skeleton(comp)
    atomisation = sum(ATOM_DHF[e] * n for e, n in comp.items())
    dh = atomisation - sum(bond_energy(b) for b in bonds)
    if name.endswith("(S)"):
        dh += rng.uniform(30.0, 50.0)  # excited singlet state above the ground state
    return dh + rng.normal(0.0, 8.0)


def _modes(comp: Dict[str, int], rng: np.random.Generator) -> Tuple[bool, List[float], int]:
    natoms = sum(comp.values())
    if natoms == 1:
        return True, [], 0
    formula = "".join(f"{e}{n if n > 1 else ''}" for e, n in sorted(comp.items()))
    linear = natoms == 2 or formula in ("CO2", "C2H2", "C2H", "CHN", "N2O")
    nmodes = 3 * natoms - (5 if linear else 6)
    bonds, _ = skeleton(comp)
    thetas: List[float] = []
    for b in bonds:
        if len(thetas) >= nmodes:
            break
        if b == ("H", "H", 1):
            thetas.append(rng.uniform(5800.0, 6300.0))
        elif "H" in b[:2]:
            thetas.append(rng.uniform(3900.0, 4700.0))
        else:
            thetas.append(rng.uniform(1300.0, 2400.0) * b[2] ** 0.4)
    while len(thetas) < nmodes:
        thetas.append(rng.uniform(500.0, 2000.0))
    sigma = 1
    if natoms == 2 and len(comp) == 1:
        sigma = 2
    elif formula in ("CO2", "C2H2", "H2O", "C2H4"):
        sigma = 2
    elif formula == "CH4":
        sigma = 12
    return linear, thetas, sigma


def cp_R(T: np.ndarray, linear: bool, natoms: int, thetas: List[float]) -> np.ndarray:
    base = 2.5 if natoms == 1 else (3.5 if linear else 4.0)
    cp = np.full_like(T, base, dtype=float)
    for th in thetas:
        x = th / T
        ex = np.exp(-x)
        cp += x * x * ex / (1.0 - ex) ** 2
    return cp


def s298_R(comp, W, linear, thetas, sigma, unpaired, rng, name) -> float:
    T = 298.15
    m = W / NA
    s_trans = math.log((2 * math.pi * m * KB * T / HPL ** 2) ** 1.5 * KB * T / P0) + 2.5
    natoms = sum(comp.values())
    s_rot = 0.0
    if natoms > 1:
        th_r = 170.0 / W ** 1.5 * rng.uniform(0.8, 1.25)
        if linear:
            s_rot = math.log(T / (sigma * th_r)) + 1.0
        else:
            th_r *= 2.0
            s_rot = math.log(math.sqrt(math.pi) / sigma * (T ** 3 / th_r ** 3) ** 0.5) + 1.5
    s_vib = 0.0
    for th in thetas:
        x = th / T
        s_vib += x / math.expm1(x) - math.log(-math.expm1(-x))
    g = 1 + unpaired
    if name.upper() == "O2":
        g = 3
    return s_trans + s_rot + s_vib + math.log(g)


def nasa7_for(name: str, rng: np.random.Generator, Tmid: float = 1000.0):
    comp = parse_formula(name)
    from .model import molar_mass
    W = molar_mass(comp)
    natoms = sum(comp.values())
    linear, thetas, sigma = _modes(comp, rng)
    _, unpaired = skeleton(comp)
    dhf = dhf_kj(name, comp, rng)  # kJ/mol
    s298 = s298_R(comp, W, linear, thetas, sigma, unpaired, rng, name)

    def fit(lo, hi):
        T = np.linspace(lo, hi, 200)
        c = cp_R(T, linear, natoms, thetas)
        V = np.vander(T / 1000.0, 5, increasing=True)
        coef, *_ = np.linalg.lstsq(V, c, rcond=None)
        return np.array([coef[k] / 1000.0 ** k for k in range(5)])

    a_lo = fit(300.0, Tmid)
    a_hi = fit(Tmid, 3500.0)
    cp_mid = float(cp_R(np.array([Tmid]), linear, natoms, thetas)[0])

    def cpv(a, T):
        return a[0] + a[1] * T + a[2] * T ** 2 + a[3] * T ** 3 + a[4] * T ** 4

    a_lo[0] += cp_mid - cpv(a_lo, Tmid)
    a_hi[0] += cp_mid - cpv(a_hi, Tmid)

    def hpoly(a, T):  # H/R without a6
        return a[0] * T + a[1] * T ** 2 / 2 + a[2] * T ** 3 / 3 + a[3] * T ** 4 / 4 + a[4] * T ** 5 / 5

    def spoly(a, T):  # S/R without a7
        return a[0] * math.log(T) + a[1] * T + a[2] * T ** 2 / 2 + a[3] * T ** 3 / 3 + a[4] * T ** 4 / 4

    a6_lo = dhf * 1000.0 / R_J - hpoly(a_lo, 298.15)
    a7_lo = s298 - spoly(a_lo, 298.15)
    a6_hi = hpoly(a_lo, Tmid) + a6_lo - hpoly(a_hi, Tmid)
    a7_hi = spoly(a_lo, Tmid) + a7_lo - spoly(a_hi, Tmid)
    low = [float(x) for x in a_lo] + [float(a6_lo), float(a7_lo)]
    high = [float(x) for x in a_hi] + [float(a6_hi), float(a7_hi)]
    return comp, W, low, high, unpaired
