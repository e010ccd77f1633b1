"""Seeded generator of synthetic, structure-matched mechanisms.

The three mechanisms the reactor is benchmarked on (LiDryer H2/O2: 9 species / 21
reactions; drm19: 21 / 84; GRI-Mech 3.0: 53 / 325) are third-party data that is not
present here. Their *shapes* are reproduced instead:

* the species lists of LiDryer and drm19 are the column headers of the reference's own
  flame fixtures (``Exec/RegTests/EB_FlamePastCylinder/pmf_040_01Atm.dat:1`` and
  ``Exec/RegTests/FlameSheet/drm19_pmf.dat:1``); the 53-species set extends the drm19
  list with formulas enumerated by this module;
* species thermo comes from :mod:`thermo_model` (physics + seed);
* reactions are element-balanced single-atom transfers ``A + B <=> C + D`` and
  recombinations ``A + B (+M) <=> C`` picked from the enumerated candidates with the
  reference mechanisms' type mix (elementary / third-body / Troe falloff), written in
  their exothermic direction with seeded Arrhenius parameters in physically plausible
  ranges; the reverse rate follows from K_c (``Model.rst:258-264``).

Every number produced here is synthetic and is labelled so wherever it is used.
"""
from __future__ import annotations

import itertools
import math
from typing import Dict, List, Tuple

import numpy as np

from .model import Arrhenius, Mechanism, Reaction, Species, R_CAL
from .thermo_model import nasa7_for, parse_formula

LIDRYER_SPECIES = ["H2", "O2", "H2O", "H", "O", "OH", "HO2", "H2O2", "N2"]
DRM19_SPECIES = ["H2", "H", "O", "O2", "OH", "H2O", "HO2", "CH2", "CH2(S)", "CH3", "CH4",
                 "CO", "CO2", "HCO", "CH2O", "CH3O", "C2H4", "C2H5", "C2H6", "N2", "AR"]
INERT = {"N2", "AR"}

# species list, reaction-type counts and the seed. Seeds are pinned so that each
# mechanism ignites a stoichiometric fuel/air mixture at 1 atm on realistic time scales
# (lidryer_syn: ~0.2 ms at 1000 K, ~10 us at 1500 K; drm19_syn and gri_syn: a few ms at 1500 K).
SHAPES = {
    "lidryer_syn": dict(species=LIDRYER_SPECIES, n_elem=14, n_tb=5, n_fo=2, n_irr=0, seed=11),
    "drm19_syn": dict(species=DRM19_SPECIES, n_elem=61, n_tb=12, n_fo=11, n_irr=2, seed=24),
    # recomb_max_dh_kcal: recombination candidates must release at least this much (bond
    # formation); the enumerated GRI-sized species set otherwise admits endothermic adducts
    # whose decomposition runs at ~1e85 /s near 300 K
    "gri_syn": dict(species=None, n_elem=284, n_tb=12, n_fo=29, n_irr=4, seed=44, recomb_max_dh_kcal=-20.0),
}

EFF_RANGES = {"H2O": (5.0, 12.0), "H2": (1.5, 2.5), "CO2": (2.0, 3.8), "CO": (1.4, 2.0),
              "CH4": (1.6, 2.4), "C2H6": (2.5, 3.2), "AR": (0.5, 0.9)}


def _formula_key(comp: Dict[str, int]) -> Tuple:
    return tuple(sorted(comp.items()))


def gri_species(rng: np.random.Generator) -> List[str]:
    """drm19 list + 32 enumerated CcHhOoNn formulas (c<=3, h<=8, o<=2, n<=1) at or below the
    saturation limit H <= 2C + N + 2."""
    from .thermo_model import skeleton
    have = {_formula_key(parse_formula(s)) for s in DRM19_SPECIES}
    cands = []
    for c, h, o, n in itertools.product(range(0, 4), range(0, 9), range(0, 3), range(0, 2)):
        comp = {k: v for k, v in (("C", c), ("H", h), ("O", o), ("N", n)) if v}
        if sum(comp.values()) < 2 or _formula_key(comp) in have:
            continue
        heavy = c + o + n
        if heavy == 0:
            continue
        if h > 2 * c + n + 2:  # above the saturation limit: no such molecule
            continue
        _, unpaired = skeleton(comp)
        if unpaired > 2:
            continue
        cands.append(comp)
    order = rng.permutation(len(cands))
    extra = []
    # prefer species with at least one C or N so the set stays hydrocarbon-like
    for i in order:
        comp = cands[i]
        if "C" not in comp and "N" not in comp:
            continue
        name = "".join(f"{e}{comp[e] if comp[e] > 1 else ''}" for e in ("C", "H", "N", "O") if e in comp)
        extra.append(name)
        if len(extra) == 32:
            break
    base = [s for s in DRM19_SPECIES if s not in INERT]
    return base + extra + ["N2", "AR"]


def _sub(a, b):
    out = dict(a)
    for k, v in b.items():
        out[k] = out.get(k, 0) - v
    return {k: v for k, v in out.items() if v != 0}


def _add(a, b):
    out = dict(a)
    for k, v in b.items():
        out[k] = out.get(k, 0) + v
    return out


def enumerate_candidates(names: List[str]):
    comps = {s: parse_formula(s) for s in names}
    react = [s for s in names if s not in INERT]
    key2names: Dict[Tuple, List[str]] = {}
    for s in react:
        key2names.setdefault(_formula_key(comps[s]), []).append(s)
    recomb = []
    for a, b in itertools.combinations_with_replacement(react, 2):
        k = _formula_key(_add(comps[a], comps[b]))
        for c in key2names.get(k, []):
            recomb.append(((a, b), (c,)))
    transfer = set()
    atoms = [{"H": 1}, {"O": 1}, {"C": 1}, {"N": 1}]
    for a, b in itertools.product(react, react):
        for x in atoms:
            ca = _sub(comps[a], x)
            if any(v < 0 for v in ca.values()) or not ca:
                continue
            db = _add(comps[b], x)
            for c in key2names.get(_formula_key(ca), []):
                for d in key2names.get(_formula_key(db), []):
                    lhs = tuple(sorted((a, b)))
                    rhs = tuple(sorted((c, d)))
                    if lhs == rhs:
                        continue
                    transfer.add(tuple(sorted((lhs, rhs))))
    return recomb, sorted(transfer)


def _dH298(sp: Dict[str, Species], lhs, rhs) -> float:
    """Reaction enthalpy at 298.15 K in units of R*K."""
    def h(s):
        a = sp[s].low
        T = 298.15
        return a[0] * T + a[1] * T ** 2 / 2 + a[2] * T ** 3 / 3 + a[3] * T ** 4 / 4 + a[4] * T ** 5 / 5 + a[5]
    return sum(h(s) for s in rhs) - sum(h(s) for s in lhs)


def _count(side) -> Dict[str, int]:
    d: Dict[str, int] = {}
    for s in side:
        d[s] = d.get(s, 0) + 1
    return d


def generate(name: str, seed: int = None) -> Mechanism:
    """Deterministic for a given (name, seed)."""
    shape = SHAPES[name]
    seed = shape["seed"] if seed is None else seed
    rng = np.random.default_rng(seed)
    names = shape["species"] or gri_species(rng)
    species = []
    radicals = {}
    for s in names:
        comp, W, low, high, unpaired = nasa7_for(s, rng)
        species.append(Species(name=s, composition=comp, W=W, Tmid=1000.0, low=low, high=high))
        radicals[s] = unpaired > 0 and s != "O2"
    sp = {s.name: s for s in species}
    elements = []
    for s in species:
        for e in s.composition:
            if e not in elements:
                elements.append(e)

    recomb, transfer = enumerate_candidates(names)
    if shape.get("recomb_max_dh_kcal") is not None:
        lim = shape["recomb_max_dh_kcal"] * 1000.0 / R_CAL  # R*K
        recomb = [c for c in recomb if _dH298(sp, c[0], c[1]) < lim]

    def score_transfer(lhs, rhs):
        dh = abs(_dH298(sp, lhs, rhs)) * 8.314e-3  # kJ/mol
        rl = sum(radicals[s] for s in lhs)
        rr = sum(radicals[s] for s in rhs)
        w = 1.0 + rl + rr
        if rl == 1 and rr == 1:
            w *= 3.0  # chain propagation (radical + molecule -> molecule + radical)
        return w * math.exp(-dh / 150.0)

    def pick(cands, n, scorer, used):
        chosen = []
        pool = [c for c in cands if c not in used]
        if n <= 0 or not pool:
            return chosen
        w = np.array([scorer(*c) for c in pool], dtype=float)
        # coverage first: make sure every reactive species appears somewhere
        covered = set()
        for c in used:
            covered.update(c[0])
            covered.update(c[1])
        reactive = [s for s in names if s not in INERT]
        for s in reactive:
            if len(chosen) >= n or s in covered:
                continue
            idx = [i for i, c in enumerate(pool) if s in c[0] or s in c[1]]
            if not idx:
                continue
            i = idx[int(np.argmax(w[idx] * rng.uniform(0.5, 1.0, len(idx))))]
            chosen.append(pool[i])
            covered.update(pool[i][0])
            covered.update(pool[i][1])
            w[i] = 0.0
        while len(chosen) < n and w.sum() > 0:
            i = int(rng.choice(len(pool), p=w / w.sum()))
            chosen.append(pool[i])
            w[i] = 0.0
        return chosen

    def recomb_score(lhs, rhs):
        return (1.0 + sum(radicals[s] for s in lhs)) * (0.2 if not all(radicals[s] for s in lhs) else 1.0)

    fo = pick(recomb, shape["n_fo"], recomb_score, [])
    tb = pick(recomb, shape["n_tb"], recomb_score, fo)
    el = pick(transfer, shape["n_elem"], score_transfer, fo + tb)

    def eff_for(rng_):
        eff = {}
        for s, (lo, hi) in EFF_RANGES.items():
            if s in sp:
                eff[s] = float(rng_.uniform(lo, hi))
        return eff

    reactions: List[Reaction] = []
    for lhs, rhs in fo:
        kinf1000 = 10 ** rng.uniform(12.8, 13.8)
        b_inf = rng.uniform(0.0, 0.6)
        k01000 = 10 ** rng.uniform(15.5, 17.5)
        b0 = rng.uniform(-2.0, -0.8)
        troe = [float(rng.uniform(0.4, 0.8)), float(10 ** rng.uniform(1.5, 2.5)),
                float(10 ** rng.uniform(3.0, 3.8))]
        if rng.uniform() < 0.5:
            troe.append(float(10 ** rng.uniform(3.6, 4.0)))
        reactions.append(Reaction(
            kind="falloff", reactants=_count(lhs), products=_count(rhs), reversible=True,
            rate=Arrhenius(kinf1000 / 1000.0 ** b_inf, b_inf, float(rng.uniform(0.0, 1000.0))),
            low=Arrhenius(k01000 / 1000.0 ** b0, b0, 0.0), troe=troe, efficiencies=eff_for(rng)))
    for lhs, rhs in tb:
        k1000 = 10 ** rng.uniform(15.0, 17.0)
        b = rng.uniform(-1.5, -0.5)
        reactions.append(Reaction(
            kind="three_body", reactants=_count(lhs), products=_count(rhs), reversible=True,
            rate=Arrhenius(k1000 / 1000.0 ** b, b, 0.0), efficiencies=eff_for(rng)))
    n_irr = shape["n_irr"]

    def closed_shell_pair(side):
        # two closed-shell (or O2) partners: such bimolecular steps have high barriers
        return all((not radicals[s]) or s == "O2" for s in side)

    for i, (lhs, rhs) in enumerate(el):
        dh = _dH298(sp, lhs, rhs)
        if dh > 0:  # write in the exothermic direction
            lhs, rhs = rhs, lhs
            dh = -dh
        k1000 = 10 ** rng.uniform(12.5, 14.0)
        b = rng.uniform(0.0, 1.5)
        ea = rng.uniform(1000.0, 12000.0)
        dh_cal = -dh * R_CAL  # endothermicity of the reverse direction, cal/mol
        if closed_shell_pair(lhs):
            ea = max(ea, rng.uniform(45000.0, 60000.0))
        if closed_shell_pair(rhs):
            ea = max(ea, rng.uniform(45000.0, 60000.0) - dh_cal)
        reactions.append(Reaction(
            kind="elementary", reactants=_count(lhs), products=_count(rhs),
            reversible=not (i < n_irr),
            rate=Arrhenius(k1000 / 1000.0 ** b, b, ea)))
    order = rng.permutation(len(reactions))
    reactions = [reactions[i] for i in order]
    return Mechanism(name=name, elements=elements, species=species, reactions=reactions,
                     synthetic=True, seed=int(seed),
                     note="SYNTHETIC structure-matched mechanism; not PelePhysics data")


def main(outdir: str) -> None:
    import os
    for name in SHAPES:
        m = generate(name)
        m.to_json(os.path.join(outdir, f"{name}.json"))
        m.to_flat(os.path.join(outdir, f"{name}.mech"))
        print(name, m.ns, m.nr)


if __name__ == "__main__":
    import os
    import sys
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(__file__), "..", "data"))
