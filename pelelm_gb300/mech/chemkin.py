"""CHEMKIN-format mechanism input (``chem.inp`` + ``therm.dat``) to and from the project's
mechanism model (:mod:`pelelm_gb300.mech.model`).

PelePhysics builds its mechanisms (``Support/Mechanism/Models/<name>``) from CHEMKIN-II inputs;
this reader takes the same inputs so a real LiDryer, drm19 or GRI-Mech 3.0 description can be
converted into the JSON the kernel generator and the oracle read:

    python -m pelelm_gb300.mech.chemkin chem.inp [therm.dat] --name drm19 --out pelelm_gb300/data

Covered (CHEMKIN-II syntax): ELEMENTS/ELEM, SPECIES/SPEC and THERMO [ALL] sections (THERMO may sit
in chem.inp or in a separate file, NASA-7 in the fixed 80-column four-line records, upper range
first); REACTIONS with its unit keywords (MOLES/MOLECULES; CAL/MOLE, KCAL/MOLE, JOULES/MOLE,
KJOULES/MOLE, KELVINS); elementary reactions; third-body reactions (+M) with efficiencies;
falloff reactions (+M) or (+species) with LOW and an optional TROE (3 or 4 parameters),
Lindemann without TROE; explicit reverse parameters REV; DUPLICATE; '!' comments; '=', '=>' and
'<=>'. Other auxiliary keywords (SRI, PLOG, CHEB, FORD, RORD, HIGH, ...) are rejected with the
reaction's line number.

Units of the model: A in (cm^3/mol)^(order-1)/s, Ea in cal/mol (the CHEMKIN defaults).
"""
from __future__ import annotations

import argparse
import os
import re
from typing import Dict, List, Optional, Tuple

from .model import ATOMIC_WEIGHT, Arrhenius, Mechanism, Reaction, Species, R_CAL

AVOGADRO = 6.02214076e23
# cal/mol per unit of each CHEMKIN activation-energy unit
_E_UNITS = {"CAL/MOLE": 1.0, "KCAL/MOLE": 1000.0, "JOULES/MOLE": 1.0 / 4.184, "KJOULES/MOLE": 1000.0 / 4.184,
            "KELVINS": R_CAL}
_UNSUPPORTED = ("SRI", "PLOG", "CHEB", "FORD", "RORD", "HIGH", "LT", "RLT", "JAN", "FIT1", "TDEP", "EXCI",
                "MOME", "XSMI", "UNITS", "USRPROG", "PCHEB", "TCHEB")


class ChemkinError(ValueError):
    pass


def _element(sym: str) -> str:
    s = sym.strip()
    return s[:1].upper() + s[1:].lower()


def _strip_comment(line: str) -> str:
    i = line.find("!")
    return line if i < 0 else line[:i]


def _sections(text: str) -> Dict[str, List[Tuple[int, str]]]:
    """Lines of each keyword section (ELEMENTS, SPECIES, THERMO, REACTIONS), with line numbers;
    the keyword line itself is kept as the first entry."""
    out: Dict[str, List[Tuple[int, str]]] = {}
    cur = None
    keys = {"ELEMENTS": "ELEMENTS", "ELEM": "ELEMENTS", "SPECIES": "SPECIES", "SPEC": "SPECIES",
            "THERMO": "THERMO", "REACTIONS": "REACTIONS", "REAC": "REACTIONS"}
    for no, raw in enumerate(text.splitlines(), 1):
        body = _strip_comment(raw) if cur != "THERMO" else raw.rstrip("\n")
        toks = body.split()
        if not toks:
            continue
        head = toks[0].upper()
        if cur is None or (cur != "THERMO" and head in keys):
            if head in keys:
                cur = keys[head]
                out.setdefault(cur, []).append((no, body))
                rest = body.split(None, 1)
                # ELEMENTS / SPECIES may list names on the keyword line itself
                if cur in ("ELEMENTS", "SPECIES") and len(rest) > 1:
                    out[cur].append((no, rest[1]))
                    if rest[1].split()[-1].upper() == "END":
                        cur = None
                continue
            raise ChemkinError(f"line {no}: text outside a section: {raw.strip()!r}")
        if head == "END" and (cur != "THERMO" or len(body.strip()) == 3):
            cur = None
            continue
        out[cur].append((no, body))
    return out


def _names(lines: List[Tuple[int, str]]) -> List[str]:
    names = []
    for _, body in lines[1:]:
        for tok in body.split():
            if tok.upper() == "END":
                return names
            names.append(tok)
    return names


def _float(s: str) -> float:
    return float(s.replace("D", "E").replace("d", "e"))


def parse_thermo(lines: List[str], wanted: Optional[List[str]] = None) -> Dict[str, Tuple[Dict[str, int], float, List[float], List[float]]]:
    """NASA-7 records: name -> (composition, Tmid, low[7], high[7]). `lines` are the THERMO
    section's lines after the keyword (the first holds the default temperature ranges)."""
    out = {}
    body = [ln.rstrip("\n") for ln in lines if ln.strip() and not ln.lstrip().startswith("!")]
    if not body:
        return out
    defaults = body[0].split()
    t_mid_default = 1000.0
    start = 0
    try:
        vals = [float(x) for x in defaults[:3]]
        if len(vals) == 3:
            t_mid_default = vals[1]
            start = 1
    except ValueError:
        start = 0
    i = start
    while i < len(body):
        l1 = body[i]
        if l1.strip().upper() == "END":
            break
        if i + 3 >= len(body):
            raise ChemkinError(f"thermo record for {l1[:18].strip()!r} is incomplete")
        l2, l3, l4 = body[i + 1], body[i + 2], body[i + 3]
        name = l1[:18].split()[0] if l1[:18].split() else ""
        comp: Dict[str, int] = {}
        for k in range(4):
            sym = l1[24 + 5 * k: 26 + 5 * k].strip()
            cnt = l1[26 + 5 * k: 29 + 5 * k].strip()
            if sym and cnt and sym != "0":
                n = int(float(cnt))
                if n:
                    comp[_element(sym)] = comp.get(_element(sym), 0) + n
        if len(l1) >= 78:
            sym, cnt = l1[73:75].strip(), l1[75:78].strip()
            if sym and cnt and sym != "0":
                n = int(float(cnt))
                if n:
                    comp[_element(sym)] = comp.get(_element(sym), 0) + n
        tmid_s = l1[65:73].strip()
        tmid = float(tmid_s) if tmid_s else t_mid_default
        coeffs = []
        for ln in (l2, l3, l4):
            for k in range(5):
                f = ln[15 * k: 15 * (k + 1)].strip()
                if f:
                    coeffs.append(_float(f))
        if len(coeffs) < 14:
            raise ChemkinError(f"thermo record for {name!r}: {len(coeffs)} coefficients, need 14")
        high, low = coeffs[:7], coeffs[7:14]
        if wanted is None or name in wanted:
            out[name] = (comp, tmid, low, high)
        i += 4
    return out


def _species_terms(side: str, species: List[str], no: int) -> Dict[str, int]:
    out: Dict[str, int] = {}
    for tok in side.split("+"):
        if not tok:
            raise ChemkinError(f"line {no}: empty species term in {side!r}")
        if tok in species:
            name, nu = tok, 1
        else:
            m = re.match(r"^(\d+)(.+)$", tok)
            if not m or m.group(2) not in species:
                raise ChemkinError(f"line {no}: unknown species {tok!r}")
            name, nu = m.group(2), int(m.group(1))
        out[name] = out.get(name, 0) + nu
    return out


def _parse_equation(eq: str, species: List[str], no: int):
    """(reactants, products, reversible, kind, falloff collider or None)."""
    s = eq.replace(" ", "")
    if "<=>" in s:
        lhs, rhs = s.split("<=>", 1)
        rev = True
    elif "=>" in s:
        lhs, rhs = s.split("=>", 1)
        rev = False
    elif "=" in s:
        lhs, rhs = s.split("=", 1)
        rev = True
    else:
        raise ChemkinError(f"line {no}: no '=', '=>' or '<=>' in {eq!r}")
    kind, coll = "elementary", None
    fm_l = re.search(r"\(\+([^)]+)\)$", lhs)
    fm_r = re.search(r"\(\+([^)]+)\)$", rhs)
    if fm_l or fm_r:
        if not (fm_l and fm_r) or fm_l.group(1).upper() != fm_r.group(1).upper():
            raise ChemkinError(f"line {no}: falloff collider must appear on both sides: {eq!r}")
        coll = fm_l.group(1)
        kind = "falloff"
        lhs, rhs = lhs[:fm_l.start()], rhs[:fm_r.start()]
        if coll.upper() == "M":
            coll = None
        elif coll not in species:
            raise ChemkinError(f"line {no}: unknown falloff collider {coll!r}")
    else:
        ml = re.search(r"\+M$", lhs, re.I)
        mr = re.search(r"\+M$", rhs, re.I)
        if ml or mr:
            if not (ml and mr):
                raise ChemkinError(f"line {no}: third body M must appear on both sides: {eq!r}")
            kind = "three_body"
            lhs, rhs = lhs[:ml.start()], rhs[:mr.start()]
    return _species_terms(lhs, species, no), _species_terms(rhs, species, no), rev, kind, coll


def read_chemkin(chem_path: str, therm_path: Optional[str] = None, name: Optional[str] = None,
                 synthetic: bool = False) -> Mechanism:
    with open(chem_path) as f:
        secs = _sections(f.read())
    if "ELEMENTS" not in secs or "SPECIES" not in secs or "REACTIONS" not in secs:
        raise ChemkinError("chem.inp needs ELEMENTS, SPECIES and REACTIONS sections")
    elements = [_element(e) for e in _names(secs["ELEMENTS"])]
    species = _names(secs["SPECIES"])
    if len(set(species)) != len(species):
        raise ChemkinError("a species is declared twice")
    thermo = {}
    if therm_path:
        with open(therm_path) as f:
            tl = f.read().splitlines()
        if tl and tl[0].split() and tl[0].split()[0].upper() == "THERMO":
            tl = tl[1:]
        thermo.update(parse_thermo(tl, species))
    if "THERMO" in secs:  # records in chem.inp take precedence
        thermo.update(parse_thermo([b for _, b in secs["THERMO"][1:]], species))
    sp_objs = []
    for s in species:
        if s not in thermo:
            raise ChemkinError(f"no thermo record for species {s!r}")
        comp, tmid, low, high = thermo[s]
        for e in comp:
            if e not in elements:
                raise ChemkinError(f"species {s!r} contains element {e!r} not in ELEMENTS")
            if e not in ATOMIC_WEIGHT:
                raise ChemkinError(f"no atomic weight for element {e!r}")
        W = sum(ATOMIC_WEIGHT[e] * n for e, n in comp.items())
        sp_objs.append(Species(name=s, composition=comp, W=W, Tmid=tmid, low=list(low), high=list(high)))

    # reactions
    head = secs["REACTIONS"][0][1].split()[1:]
    e_unit, molecules = 1.0, False
    for tok in head:
        t = tok.upper()
        if t in _E_UNITS:
            e_unit = _E_UNITS[t]
        elif t == "MOLECULES":
            molecules = True
        elif t == "MOLES":
            molecules = False
        else:
            raise ChemkinError(f"REACTIONS: unsupported unit keyword {tok!r}")
    reactions: List[Reaction] = []
    line_of: List[int] = []
    pending: Optional[dict] = None

    def arr(vals, order):
        A = vals[0] * (AVOGADRO ** (order - 1) if molecules else 1.0)
        return Arrhenius(A=A, beta=vals[1], Ea=vals[2] * e_unit)

    def flush():
        nonlocal pending
        if pending is None:
            return
        p = pending
        order = sum(p["reactants"].values())
        third = 1 if p["kind"] == "three_body" else 0
        rate = arr(p["arr"], order + third)
        low = None
        if p["kind"] == "falloff":
            if p.get("low") is None:
                raise ChemkinError(f"line {p['no']}: falloff reaction without LOW")
            low = arr(p["low"], order + 1)
        elif p.get("low") is not None or p.get("troe") is not None:
            raise ChemkinError(f"line {p['no']}: LOW/TROE on a reaction without (+M)")
        rev = None
        if p.get("rev") is not None:
            if not p["reversible"]:
                raise ChemkinError(f"line {p['no']}: REV on an irreversible reaction")
            if p["kind"] == "falloff":
                raise ChemkinError(f"line {p['no']}: REV on a falloff reaction is not supported")
            rev = arr(p["rev"], sum(p["products"].values()) + third)
        eff = dict(p.get("eff", {}))
        if p["coll"] is not None:  # (+species): only that species collides
            if eff:
                raise ChemkinError(f"line {p['no']}: efficiencies with a specific falloff collider")
            eff = {s: (1.0 if s == p["coll"] else 0.0) for s in species}
        if eff and p["kind"] == "elementary":
            raise ChemkinError(f"line {p['no']}: third-body efficiencies on a reaction without M")
        reactions.append(Reaction(kind=p["kind"], reactants=p["reactants"], products=p["products"],
                                  reversible=p["reversible"], rate=rate, low=low,
                                  troe=list(p["troe"]) if p.get("troe") is not None else None,
                                  efficiencies=eff, rev=rev, duplicate=p.get("dup", False)))
        line_of.append(p["no"])
        pending = None

    num = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eEdD][-+]?\d+)?"
    for no, body in secs["REACTIONS"][1:]:
        text = body.strip()
        if not text:
            continue
        up = text.upper()
        toks = text.split()
        is_rx = ("=" in text) and len(toks) >= 4 and all(re.fullmatch(num, t) for t in toks[-3:])
        if is_rx:
            flush()
            eq = " ".join(toks[:-3])
            rs, ps, rev, kind, coll = _parse_equation(eq, species, no)
            pending = {"no": no, "reactants": rs, "products": ps, "reversible": rev, "kind": kind, "coll": coll,
                       "arr": [_float(t) for t in toks[-3:]]}
            continue
        if pending is None:
            raise ChemkinError(f"line {no}: auxiliary data before any reaction: {text!r}")
        if up.startswith("DUP"):
            pending["dup"] = True
            continue
        for kw in _UNSUPPORTED:
            if re.match(rf"^{kw}\b", up):
                raise ChemkinError(f"line {no}: auxiliary keyword {kw} is not supported")
        m = re.match(r"^(LOW|TROE|REV)\s*/(.*)/\s*$", text, re.I)
        if m:
            vals = [_float(v) for v in m.group(2).split()]
            key = m.group(1).lower()
            if key in ("low", "rev") and len(vals) != 3:
                raise ChemkinError(f"line {no}: {key.upper()} needs 3 values")
            if key == "troe" and len(vals) not in (3, 4):
                raise ChemkinError(f"line {no}: TROE needs 3 or 4 values")
            pending[key] = vals
            continue
        # third-body efficiencies: NAME/value/ pairs
        pairs = re.findall(r"([^\s/]+)\s*/\s*(" + num + r")\s*/", text)
        rest = re.sub(r"([^\s/]+)\s*/\s*(" + num + r")\s*/", "", text).strip()
        if not pairs or rest:
            raise ChemkinError(f"line {no}: cannot read {text!r}")
        for sname, v in pairs:
            if sname not in species:
                raise ChemkinError(f"line {no}: efficiency for unknown species {sname!r}")
            pending.setdefault("eff", {})[sname] = _float(v)
    flush()
    # DUPLICATE pairs: each marked reaction needs a partner with the same stoichiometry
    for j, r in enumerate(reactions):
        same = [k for k, o in enumerate(reactions) if k != j and o.reactants == r.reactants
                and o.products == r.products and o.kind == r.kind]
        if r.duplicate and not any(reactions[k].duplicate for k in same):
            raise ChemkinError(f"line {line_of[j]}: DUPLICATE without a duplicate partner")
        if same and not r.duplicate:
            raise ChemkinError(f"line {line_of[j]}: reaction repeated without DUPLICATE")
    nm = name or os.path.splitext(os.path.basename(chem_path))[0]
    return Mechanism(name=nm, elements=elements, species=sp_objs, reactions=reactions, synthetic=synthetic,
                     note=f"read from CHEMKIN input {os.path.basename(chem_path)}")


# ---------------------------------------------------------------------------- writer
def _fmt_thermo_record(s: Species, tlow: float = 300.0, thigh: float = 5000.0) -> List[str]:
    comp = list(s.composition.items())
    if len(comp) > 5:
        raise ChemkinError(f"species {s.name}: more than 5 elements")
    field = ""
    for k in range(4):
        if k < len(comp):
            e, n = comp[k]
            field += f"{e.upper():<2}{n:>3d}"
        else:
            field += " " * 5
    l1 = f"{s.name:<18}{'':6}{field}G{tlow:10.3f}{thigh:10.3f}{s.Tmid:8.2f}"
    if len(comp) == 5:
        e, n = comp[4]
        l1 += f"{e.upper():<2}{n:>3d}"
    l1 = f"{l1:<79}1"
    c = list(s.high) + list(s.low)
    fmt = lambda v: f"{v:15.8E}"
    l2 = "".join(fmt(v) for v in c[0:5]) + "    2"
    l3 = "".join(fmt(v) for v in c[5:10]) + "    3"
    l4 = "".join(fmt(v) for v in c[10:14]) + " " * 15 + "    4"
    return [l1, l2, l3, l4]


def write_chemkin(m: Mechanism, chem_path: str, therm_path: Optional[str] = None) -> None:
    """chem.inp (and therm.dat, else a THERMO section inside chem.inp) in CHEMKIN-II syntax;
    reaction parameters with full double precision, thermo in the fixed format's E15.8."""
    out = ["ELEMENTS", " ".join(e.upper() for e in m.elements), "END", "SPECIES"]
    line = ""
    for s in m.species:
        if len(line) + len(s.name) + 1 > 70:
            out.append(line.rstrip())
            line = ""
        line += s.name + " "
    out += [line.rstrip(), "END"]
    therm = ["THERMO ALL", "   300.000  1000.000  5000.000"]
    for s in m.species:
        therm += _fmt_thermo_record(s)
    therm.append("END")
    if therm_path is None:
        out += therm
    out.append("REACTIONS  CAL/MOLE  MOLES")

    def side(d, tail):
        return "+".join((f"{n}" if n > 1 else "") + s for s, n in d.items()) + tail

    for r in m.reactions:
        tail = {"elementary": "", "three_body": "+M", "falloff": "(+M)"}[r.kind]
        arrow = "<=>" if r.reversible else "=>"
        eq = side(r.reactants, tail) + arrow + side(r.products, tail)
        out.append(f"{eq:<40} {r.rate.A!r} {r.rate.beta!r} {r.rate.Ea!r}")
        if r.kind == "falloff":
            out.append(f"    LOW / {r.low.A!r} {r.low.beta!r} {r.low.Ea!r} /")
            if r.troe:
                out.append("    TROE / " + " ".join(repr(float(t)) for t in r.troe) + " /")
        if r.rev is not None:
            out.append(f"    REV / {r.rev.A!r} {r.rev.beta!r} {r.rev.Ea!r} /")
        if r.efficiencies:
            out.append("    " + " ".join(f"{s}/{v!r}/" for s, v in r.efficiencies.items()))
        if r.duplicate:
            out.append("    DUPLICATE")
    out.append("END")
    with open(chem_path, "w") as f:
        f.write("\n".join(out) + "\n")
    if therm_path is not None:
        with open(therm_path, "w") as f:
            f.write("\n".join(therm) + "\n")


def main(argv=None):
    p = argparse.ArgumentParser(description="CHEMKIN mechanism -> pelelm_gb300 mechanism JSON and oracle input")
    p.add_argument("chem")
    p.add_argument("therm", nargs="?")
    p.add_argument("--name", required=True)
    p.add_argument("--out", default=os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data"))
    a = p.parse_args(argv)
    m = read_chemkin(a.chem, a.therm, name=a.name)
    os.makedirs(a.out, exist_ok=True)
    m.to_json(os.path.join(a.out, f"{a.name}.json"))
    m.to_flat(os.path.join(a.out, f"{a.name}.mech"))
    print(f"{a.name}: {m.ns} species, {m.nr} reactions -> {a.out}")


if __name__ == "__main__":
    main()
