"""Mechanism data model: species (composition, molar mass, NASA-7 thermo) and reactions
(elementary, third-body, Lindemann/Troe falloff) in CHEMKIN units.

This is the project's mechanism description format. It carries the same information a
CHEMKIN input / PelePhysics ``Support/Mechanism/Models/<name>/mechanism.{H,cpp}`` encodes:
the kinetics and thermo equations are those of ``Docs/source/manual/Model.rst:227-296``
(modified Arrhenius, K_c from NASA-7 Gibbs energies, third-body and falloff
specialisations).

Units (CHEMKIN/CGS): A in (cm^3/mol)^(order-1)/s, Ea in cal/mol, W in g/mol, T in K.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field, asdict
from typing import Dict, List, Optional

R_CAL = 1.98720425864083  # cal/mol/K
R_ERG = 8.31446261815324e7  # erg/mol/K
P_ATM = 1.01325e6  # dyn/cm^2

ATOMIC_WEIGHT = {"H": 1.008, "C": 12.011, "N": 14.007, "O": 15.999, "Ar": 39.95, "He": 4.0026}


@dataclass
class Species:
    name: str
    composition: Dict[str, int]
    W: float
    Tmid: float
    low: List[float]   # NASA-7 a1..a7 for T < Tmid
    high: List[float]  # NASA-7 a1..a7 for T >= Tmid


@dataclass
class Arrhenius:
    A: float
    beta: float
    Ea: float  # cal/mol


@dataclass
class Reaction:
    kind: str  # "elementary" | "three_body" | "falloff"
    reactants: Dict[str, int]
    products: Dict[str, int]
    reversible: bool
    rate: Arrhenius                      # k (elementary/three-body) or k_inf (falloff)
    low: Optional[Arrhenius] = None      # k_0 (falloff)
    troe: Optional[List[float]] = None   # [alpha, T3, T1] or [alpha, T3, T1, T2]; None => Lindemann
    efficiencies: Dict[str, float] = field(default_factory=dict)  # third-body (default 1)
    rev: Optional[Arrhenius] = None      # explicit reverse Arrhenius (CHEMKIN REV); None => K_c
    duplicate: bool = False              # CHEMKIN DUPLICATE marker (no kinetic effect)

    def equation(self) -> str:
        def side(d):
            return " + ".join((f"{n} " if n > 1 else "") + s for s, n in d.items())
        m = {"elementary": "", "three_body": " + M", "falloff": " (+M)"}[self.kind]
        arrow = " <=> " if self.reversible else " => "
        return side(self.reactants) + m + arrow + side(self.products) + m


@dataclass
class Mechanism:
    name: str
    elements: List[str]
    species: List[Species]
    reactions: List[Reaction]
    synthetic: bool = True
    seed: int = 0
    note: str = ""

    @property
    def ns(self) -> int:
        return len(self.species)

    @property
    def nr(self) -> int:
        return len(self.reactions)

    def index(self, name: str) -> int:
        for i, s in enumerate(self.species):
            if s.name == name:
                return i
        raise KeyError(name)

    # ---------------------------------------------------------------- io
    def to_json(self, path: str) -> None:
        with open(path, "w") as f:
            json.dump(asdict(self), f, indent=1)

    @staticmethod
    def from_json(path: str) -> "Mechanism":
        with open(path) as f:
            d = json.load(f)
        sp = [Species(**s) for s in d["species"]]
        rx = []
        for r in d["reactions"]:
            r = dict(r)
            r["rate"] = Arrhenius(**r["rate"])
            if r.get("low") is not None:
                r["low"] = Arrhenius(**r["low"])
            if r.get("rev") is not None:
                r["rev"] = Arrhenius(**r["rev"])
            rx.append(Reaction(**r))
        return Mechanism(name=d["name"], elements=d["elements"], species=sp, reactions=rx,
                         synthetic=d.get("synthetic", True), seed=d.get("seed", 0),
                         note=d.get("note", ""))

    def to_flat(self, path: str) -> None:
        """Whitespace-separated numeric dump read by the C++ oracle (no JSON parser there).

        Layout:
          ns nr nel
          per species: W Tmid low[7] high[7] ncomp (el_index count)*
          per reaction: kind(0/1/2) reversible nreac (sp nu)* nprod (sp nu)* A beta Ea
                        [falloff: A0 beta0 Ea0 ntroe troe*] [third-body/falloff: neff (sp eff)*]
        """
        el_idx = {e: i for i, e in enumerate(self.elements)}
        kinds = {"elementary": 0, "three_body": 1, "falloff": 2}
        for j, r in enumerate(self.reactions):
            if r.rev is not None:
                raise ValueError(f"reaction {j} ({r.equation()}): explicit reverse Arrhenius parameters "
                                 "(REV) are not supported by the rate kernels; reverse rates come from K_c")
        out = [f"{self.ns} {self.nr} {len(self.elements)}"]
        for s in self.species:
            comp = " ".join(f"{el_idx[e]} {n}" for e, n in s.composition.items())
            out.append(f"{s.W!r} {s.Tmid!r} " + " ".join(repr(float(a)) for a in s.low) + " "
                       + " ".join(repr(float(a)) for a in s.high) + f" {len(s.composition)} {comp}")
        for r in self.reactions:
            toks = [str(kinds[r.kind]), str(int(r.reversible))]
            toks.append(str(len(r.reactants)))
            for sname, nu in r.reactants.items():
                toks += [str(self.index(sname)), str(nu)]
            toks.append(str(len(r.products)))
            for sname, nu in r.products.items():
                toks += [str(self.index(sname)), str(nu)]
            toks += [repr(float(r.rate.A)), repr(float(r.rate.beta)), repr(float(r.rate.Ea))]
            if r.kind == "falloff":
                toks += [repr(float(r.low.A)), repr(float(r.low.beta)), repr(float(r.low.Ea))]
                troe = r.troe or []
                toks.append(str(len(troe)))
                toks += [repr(float(t)) for t in troe]
            if r.kind in ("three_body", "falloff"):
                toks.append(str(len(r.efficiencies)))
                for sname, e in r.efficiencies.items():
                    toks += [str(self.index(sname)), repr(float(e))]
            out.append(" ".join(toks))
        with open(path, "w") as f:
            f.write("\n".join(out) + "\n")


def molar_mass(comp: Dict[str, int]) -> float:
    return sum(ATOMIC_WEIGHT[e] * n for e, n in comp.items())
